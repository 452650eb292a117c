// Host-side decode planner.
//
// OpenZL's universal decoder (src/openzl/decompress/decompress2.c:1266-1290,
// runDecoders/processStream) walks a frame's decoder list serially, creating
// each regenerated stream when its decoder runs. On the GPU the same walk is
// done once on the host, before any payload is touched: every stream's type,
// width and element count follows from the frame headers and codec headers
// alone (the one exception, the FSE normalized-count header, is parsed here
// from the stored stream). The planner then
//   1. fuses numeric chains (delta <- zigzag <- view <- transpose|bitpack) into
//      one pipeline task,
//   2. places streams: outputs of views and concatenations (splitN) are laid
//      directly where their consumer wants them, so those decoders cost no
//      copy, and the last decoder writes straight into the caller's buffer,
//   3. assigns dependency levels and groups tasks per (level, codec kind),
//      one kernel launch per group across all frames of a batch.
#include "dec_plan.h"

#include <algorithm>
#include <cstring>
#include <functional>
#include <iterator>
#include <thread>
#include <type_traits>
#include <unordered_map>

namespace ozl {

namespace {

// Standard transform IDs (src/openzl/common/wire_format.h:211-306).
enum : uint32_t {
    T_DELTA = 1,
    T_ZIGZAG = 3,
    T_TSPLIT = 4,
    T_CONV_SERIAL_TO_STRUCT = 5,
    T_CONV_STRUCT_TO_SERIAL = 6,
    T_CONV_STRUCT_TO_NUM = 7,
    T_CONV_NUM_TO_STRUCT = 8,
    T_CONV_SERIAL_TO_NUM = 9,
    T_CONV_NUM_TO_SERIAL = 10,
    T_SEP_STRING = 12,
    T_BITPACK_SERIAL = 27,
    T_BITPACK_INT = 28,
    T_FLATPACK = 29,
    T_FLOATDEC = 33,
    T_TOKENIZE_FIXED = 36,
    T_TOKENIZE_NUMERIC = 37,
    T_SPLITN = 40,
    T_CONST_SERIAL = 44,
    T_CONST_FIXED = 45,
    T_SPLITN_STRUCT = 47,
    T_SPLITN_NUM = 48,
    T_FSE = 49,
    T_HUF = 50,
    T_HUF16 = 51,
    T_NCOUNT = 52,
    T_ID_END = 63,
};

enum : int { TY_SERIAL = 1, TY_STRUCT = 2, TY_NUMERIC = 4, TY_STRING = 8 };

// Decoder signature: singleton inputs (types in decoder order), variable
// input type, regenerated type. Mirrors the graph descriptions registered in
// src/openzl/codecs/decoder_registry.c:88-161.
struct Sig {
    bool known;
    int nbSO;
    int so[2];
    int vo;
    int out;
    bool view;    // regenerated bytes equal the input bytes
    bool concat;  // regenerated stream is the concatenation of the inputs
};

Sig signature(uint32_t id)
{
    switch (id) {
        case T_DELTA:
        case T_ZIGZAG: return { true, 1, { TY_NUMERIC, 0 }, 0, TY_NUMERIC, false, false };
        case T_TSPLIT: return { true, 0, { 0, 0 }, TY_SERIAL, TY_STRUCT, false, false };
        case T_CONV_SERIAL_TO_STRUCT: return { true, 1, { TY_STRUCT, 0 }, 0, TY_SERIAL, true, false };
        // separate_string_components (graph_conversion.h:61-66): content, lengths -> string
        case T_SEP_STRING: return { true, 2, { TY_SERIAL, TY_NUMERIC }, 0, TY_STRING, false, false };
        case T_CONV_STRUCT_TO_SERIAL: return { true, 1, { TY_SERIAL, 0 }, 0, TY_STRUCT, true, false };
        case T_CONV_STRUCT_TO_NUM: return { true, 1, { TY_NUMERIC, 0 }, 0, TY_STRUCT, true, false };
        case T_CONV_NUM_TO_STRUCT: return { true, 1, { TY_STRUCT, 0 }, 0, TY_NUMERIC, true, false };
        case T_CONV_SERIAL_TO_NUM: return { true, 1, { TY_NUMERIC, 0 }, 0, TY_SERIAL, true, false };
        case T_CONV_NUM_TO_SERIAL: return { true, 1, { TY_SERIAL, 0 }, 0, TY_NUMERIC, true, false };
        case T_BITPACK_SERIAL: return { true, 1, { TY_SERIAL, 0 }, 0, TY_SERIAL, false, false };
        case T_BITPACK_INT: return { true, 1, { TY_SERIAL, 0 }, 0, TY_NUMERIC, false, false };
        case T_FLATPACK: return { true, 2, { TY_SERIAL, TY_SERIAL }, 0, TY_SERIAL, false, false };
        case T_FLOATDEC: return { true, 2, { TY_STRUCT, TY_SERIAL }, 0, TY_NUMERIC, false, false };
        case T_TOKENIZE_FIXED: return { true, 2, { TY_STRUCT, TY_NUMERIC }, 0, TY_STRUCT, false, false };
        case T_TOKENIZE_NUMERIC: return { true, 2, { TY_NUMERIC, TY_NUMERIC }, 0, TY_NUMERIC, false, false };
        case T_SPLITN: return { true, 0, { 0, 0 }, TY_SERIAL, TY_SERIAL, false, true };
        case T_SPLITN_STRUCT: return { true, 0, { 0, 0 }, TY_STRUCT, TY_STRUCT, false, true };
        case T_SPLITN_NUM: return { true, 0, { 0, 0 }, TY_NUMERIC, TY_NUMERIC, false, true };
        case T_CONST_SERIAL: return { true, 1, { TY_SERIAL, 0 }, 0, TY_SERIAL, false, false };
        case T_CONST_FIXED: return { true, 1, { TY_STRUCT, 0 }, 0, TY_STRUCT, false, false };
        case T_FSE:
        case T_HUF: return { true, 2, { TY_NUMERIC, TY_SERIAL }, 0, TY_SERIAL, false, false };
        case T_HUF16: return { true, 2, { TY_NUMERIC, TY_SERIAL }, 0, TY_STRUCT, false, false };
        case T_NCOUNT: return { true, 1, { TY_SERIAL, 0 }, 0, TY_NUMERIC, false, false };
        default: return { false, 0, { 0, 0 }, 0, 0, false, false };
    }
}

// ZL error codes used by the planner (include/openzl/zl_errors_types.h).
enum : int {
    E_GENERIC = 1,
    E_SRC_SMALL = 3,
    E_DST_SMALL = 5,
    E_HEADER = 10,
    E_CORRUPT = 12,
    E_CK_COMPRESSED = 13,
    E_VERSION = 60,
    E_LIMIT = 81,
    E_TRANSFORM = 32,
};

struct Reader {
    const uint8_t* p;
    const uint8_t* end;
    bool varint(uint64_t& v)
    {
        v = 0;
        for (int sh = 0; sh < 70; sh += 7) {
            if (p >= end) return false;
            uint8_t b = *p++;
            v |= uint64_t(b & 0x7f) << sh;
            if (!(b & 0x80)) return true;
        }
        return false;
    }
    // n fields of nbBits, LSB-first (frame-header bit-packed arrays).
    bool unpack(std::vector<uint64_t>& dst, size_t n, int nbBits)
    {
        size_t need = (n * size_t(nbBits) + 7) / 8;
        if (size_t(end - p) < need) return false;
        dst.assign(n, 0);
        for (size_t i = 0; i < n; i++) {
            size_t bit = i * size_t(nbBits);
            uint64_t v = 0;
            for (int b = 0; b < nbBits; b++) {
                size_t q = bit + size_t(b);
                v |= uint64_t((p[q >> 3] >> (q & 7)) & 1) << b;
            }
            dst[i] = v;
        }
        p += need;
        return true;
    }
};

int nextPow2Bits(uint64_t v)
{
    int n = 0;
    while (n < 64 && (uint64_t(1) << n) < v) n++;
    return n;
}

uint64_t readLEn(const uint8_t* p, size_t n)
{
    uint64_t v = 0;
    for (size_t i = 0; i < n; i++) v |= uint64_t(p[i]) << (8 * i);
    return v;
}

uint32_t readLE32(const uint8_t* p) { return uint32_t(readLEn(p, 4)); }

int highbit32(uint32_t v) { return 31 - __builtin_clz(v); }

// FSE normalized-count header parser (the format of
// src/openzl/fse/common/entropy_common.c:42-185). Returns bytes consumed or -1.
long parseNCount(int16_t* norm, unsigned& nbSym, const uint8_t* src, size_t size)
{
    size_t pos = 0;
    size_t const total = size * 8;
    auto bits = [&](int nb) -> uint32_t {
        uint32_t v = 0;
        for (int i = 0; i < nb; i++) {
            size_t q = pos + size_t(i);
            if (q < total) v |= uint32_t((src[q >> 3] >> (q & 7)) & 1) << i;
        }
        return v;
    };
    if (size == 0) return -1;
    int nb = int(bits(4)) + 5;
    pos += 4;
    if (nb > 15) return -1;
    int remaining = (1 << nb) + 1, threshold = 1 << nb;
    nb++;
    unsigned sym = 0;
    bool prev0 = false;
    std::memset(norm, 0, 256 * sizeof(int16_t));
    while (remaining > 1 && sym < 256) {
        if (prev0) {
            unsigned z = sym;
            while (bits(2) == 3) { z += 3; pos += 2; }
            z += bits(2);
            pos += 2;
            if (z > 256) return -1;
            sym = z;
            if (sym >= 256) break;
        }
        int const max = (2 * threshold - 1) - remaining;
        uint32_t const low = bits(nb - 1);
        int count;
        if (int(low) < max) {
            count = int(low);
            pos += size_t(nb - 1);
        } else {
            count = int(bits(nb));
            if (count >= threshold) count -= max;
            pos += size_t(nb);
        }
        count--;
        remaining -= count < 0 ? -count : count;
        norm[sym++] = int16_t(count);
        prev0 = (count == 0);
        while (remaining < threshold) {
            nb--;
            threshold >>= 1;
        }
    }
    if (remaining != 1 || sym > 256 || pos > total) return -1;
    nbSym = sym;
    return long((pos + 7) / 8);
}

} // namespace

// ---------------------------------------------------------------------------
int DecodePlan::build(size_t nbFrames, const uint8_t* const* hFrames, const size_t* frameSizes,
                      const size_t* dstCapacities, bool ckContent, bool ckCompressed,
                      std::string& err)
{
    frames.assign(nbFrames, FramePlan());
    streams.clear();
    nodes.clear();
    hashes.clear();
    directCopies.clear();
    gathers.clear();
    widens.clear();
    params.clear();
    arenaBytes = 0;
    totalOut = 0;
    for (size_t f = 0; f < nbFrames; f++) {
        int rc = planFrame(int(f), hFrames[f], frameSizes[f],
                           dstCapacities ? dstCapacities[f] : SIZE_MAX, ckContent, ckCompressed, err);
        if (rc) {
            err = "frame " + std::to_string(f) + ": " + err;
            return rc;
        }
        totalOut += frames[f].decodedSize;
    }
    return 0;
}

int DecodePlan::buildParallel(size_t nbFrames, const uint8_t* const* hFrames, const size_t* frameSizes,
                              const size_t* dstCapacities, bool ckContent, bool ckCompressed, std::string& err,
                              unsigned threads)
{
    constexpr size_t kMinFrames = 64; // frames per thread below which threads do not pay
    size_t const T = std::min<size_t>(threads, nbFrames / kMinFrames);
    if (T < 2) return build(nbFrames, hFrames, frameSizes, dstCapacities, ckContent, ckCompressed, err);
    // runs of about equal compressed bytes
    uint64_t total = 0;
    for (size_t f = 0; f < nbFrames; f++) total += frameSizes[f];
    std::vector<size_t> first{ 0 };
    uint64_t acc = 0;
    for (size_t f = 0; f + 1 < nbFrames && first.size() < T; f++) {
        acc += frameSizes[f];
        if (acc * T >= total * first.size()) first.push_back(f + 1);
    }
    first.push_back(nbFrames);
    size_t const runs = first.size() - 1;
    std::vector<DecodePlan> sub(runs);
    std::vector<int> rc(runs, 0);
    std::vector<std::string> errs(runs);
    auto one = [&](size_t t) {
        size_t const f0 = first[t];
        rc[t] = sub[t].build(first[t + 1] - f0, hFrames + f0, frameSizes + f0, dstCapacities ? dstCapacities + f0 : nullptr,
                             ckContent, ckCompressed, errs[t]);
    };
    std::vector<std::thread> th;
    for (size_t t = 1; t < runs; t++) th.emplace_back(one, t);
    one(0);
    for (std::thread& x : th) x.join();
    for (size_t t = 0; t < runs; t++)
        if (rc[t]) return build(nbFrames, hFrames, frameSizes, dstCapacities, ckContent, ckCompressed, err);
    // join
    frames.clear();
    streams.clear();
    nodes.clear();
    hashes.clear();
    directCopies.clear();
    gathers.clear();
    widens.clear();
    params.clear();
    arenaBytes = 0;
    totalOut = 0;
    for (size_t t = 0; t < runs; t++) {
        DecodePlan& P = sub[t];
        int const fo = int(first[t]), so = int(streams.size()), no = int(nodes.size());
        uint64_t const ao = arenaBytes;                         // 64-byte multiple
        uint64_t const po = (params.size() + 15) & ~size_t(15); // the next 16-byte aligned block
        for (PlanStream& x : P.streams) {
            if (x.producer >= 0) x.producer += no;
            if (x.parent >= 0) x.parent += so;
            if (x.lens >= 0) x.lens += so;
            if (x.frame >= 0) x.frame += fo;
            if (x.loc == L_ARENA) x.off += ao;
            else if (x.loc == L_PARAM) x.off += po;
        }
        for (PlanNode& x : P.nodes) {
            for (int& i : x.ins) i += so;
            if (x.out >= 0) x.out += so;
            if (x.frame >= 0) x.frame += fo;
            x.paramOff += po;
        }
        for (PlanHash& x : P.hashes) {
            x.frame += fo;
            if (x.where == HW_ARENA) x.off += ao;
        }
        for (PlanCopy& x : P.directCopies) x.frame += fo;
        for (PlanGather& x : P.gathers) {
            x.frame += fo;
            x.arenaOff += ao;
        }
        for (PlanWiden& x : P.widens) {
            x.stream += so;
            x.frame += fo;
        }
        frames.insert(frames.end(), std::make_move_iterator(P.frames.begin()), std::make_move_iterator(P.frames.end()));
        streams.insert(streams.end(), P.streams.begin(), P.streams.end());
        nodes.insert(nodes.end(), std::make_move_iterator(P.nodes.begin()), std::make_move_iterator(P.nodes.end()));
        hashes.insert(hashes.end(), P.hashes.begin(), P.hashes.end());
        directCopies.insert(directCopies.end(), P.directCopies.begin(), P.directCopies.end());
        gathers.insert(gathers.end(), P.gathers.begin(), P.gathers.end());
        widens.insert(widens.end(), P.widens.begin(), P.widens.end());
        if (!P.params.empty()) {
            params.resize(po);
            params.insert(params.end(), P.params.begin(), P.params.end());
        }
        arenaBytes += P.arenaBytes;
        totalOut += P.totalOut;
    }
    return 0;
}

// Frame header. Versions 21+ open with a flags byte and store the output
// count, types and varint sizes after it (decode_frameheader.c:94-107,
// 148-173, 193-250, 270-370); versions 8..20 pack the count and types into
// byte 4 onwards, store LE32 sizes and keep the checksum flags in the block
// header (decode_frameheader.c:58-92, 110-147, 177-190).
int parseFrameHeader(const uint8_t* src, size_t size, FrameHeader& h, std::string& err)
{
    h = FrameHeader();
    if (size < 8) { err = "frame too small"; return E_SRC_SMALL; }
    uint32_t const magic = readLE32(src);
    // ZL_MIN_FORMAT_VERSION .. ZL_MAX_FORMAT_VERSION (include/openzl/zl_version.h:49-57)
    if (magic < 0xD7B1A5C0u + 8 || magic > 0xD7B1A5C0u + 23) {
        err = "unsupported format version or bad magic";
        return E_VERSION;
    }
    unsigned const version = magic - 0xD7B1A5C0u;
    h.version = version;
    static const int typeMap[4] = { TY_SERIAL, TY_STRUCT, TY_NUMERIC, TY_STRING };
    size_t nbOut = 1, pos = 4;
    auto byteAt = [&](size_t i, uint8_t& v) -> bool {
        if (i >= size) return false;
        v = src[i];
        return true;
    };
    if (version < 21) {
        if (version >= 15) {
            uint8_t t;
            if (size < pos + 1 + 4 || !byteAt(pos++, t)) { err = "truncated frame header"; return E_SRC_SMALL; }
            nbOut = size_t(t >> 6) + 1;
            if (nbOut == 4) {
                if (!byteAt(pos++, t)) { err = "truncated frame header"; return E_SRC_SMALL; }
                nbOut = size_t(t >> 4) + 4;
            }
            if (nbOut == 19) {
                if (!byteAt(pos++, t)) { err = "truncated frame header"; return E_SRC_SMALL; }
                nbOut = size_t(t) + 19;
            }
            if (nbOut == 274) {
                if (pos + 2 > size) { err = "truncated frame header"; return E_SRC_SMALL; }
                nbOut = size_t(src[pos] | (src[pos + 1] << 8)) + 274;
                pos += 2;
            }
        } else if (version == 14) {
            pos++; // the type byte
        }
        if (nbOut > 2048) { err = "too many outputs"; return E_LIMIT; }
        h.types.assign(nbOut, TY_SERIAL);
        if (version >= 14) {
            for (size_t n = 0; n < nbOut && n < 3; n++) h.types[n] = typeMap[(src[4] >> (2 * n)) & 3];
            if (nbOut > 3) {
                if (size < 6) { err = "truncated frame header"; return E_SRC_SMALL; }
                for (size_t n = 3; n < nbOut && n < 5; n++) h.types[n] = typeMap[(src[5] >> (2 * (n - 3))) & 3];
            }
            uint8_t tok = 0;
            for (size_t n = 5; n < nbOut; n++) {
                size_t const sh = ((n - 5) % 4) * 2;
                if (sh == 0 && !byteAt(pos++, tok)) { err = "truncated frame header"; return E_SRC_SMALL; }
                h.types[n] = typeMap[(tok >> sh) & 3];
            }
        }
        if (pos + 4 * nbOut > size) { err = "truncated frame header"; return E_SRC_SMALL; }
        h.sizes.resize(nbOut);
        for (size_t n = 0; n < nbOut; n++) h.sizes[n] = readLE32(src + pos + 4 * n);
        h.end = pos + 4 * nbOut;
        h.nbStrings.assign(nbOut, 0);
        for (int t : h.types)
            if (t == TY_STRING) { err = "string outputs before format version 21"; return E_LIMIT; }
    } else {
        if (size < 9) { err = "frame too small"; return E_SRC_SMALL; }
        uint8_t const flags = src[4];
        h.hasContentCk = flags & 1;
        h.hasCompressedCk = (flags >> 1) & 1;
        bool const hasComment = (flags >> 2) & 1;
        uint8_t const t1 = src[5];
        pos = 6;
        nbOut = t1 & 15;
        size_t done = 0;
        if (nbOut == 15) {
            uint8_t t2;
            if (!byteAt(pos++, t2)) { err = "truncated frame header"; return E_SRC_SMALL; }
            nbOut = (size_t(t2) << 4) + (t1 >> 4) + 15;
        }
        if (nbOut == 0) { err = "frame without outputs"; return E_CORRUPT; }
        if (nbOut > 2048) { err = "too many outputs"; return E_LIMIT; }
        h.types.assign(nbOut, TY_SERIAL);
        if ((t1 & 15) != 15) {
            for (size_t n = 0; n < nbOut && n < 2; n++) h.types[n] = typeMap[(t1 >> (4 + 2 * n)) & 3];
            done = 2;
        }
        uint8_t tok = 0;
        for (size_t n = done; n < nbOut; n++) {
            size_t const sh = ((n - done) % 4) * 2;
            if (sh == 0 && !byteAt(pos++, tok)) { err = "truncated frame header"; return E_SRC_SMALL; }
            h.types[n] = typeMap[(tok >> sh) & 3];
        }
        Reader rd{ src + pos, src + size };
        h.sizes.resize(nbOut);
        for (size_t n = 0; n < nbOut; n++) {
            uint64_t sz1;
            if (!rd.varint(sz1)) { err = "truncated frame header"; return E_SRC_SMALL; }
            if (sz1 == 0) { err = "unknown decompressed size"; return E_LIMIT; }
            h.sizes[n] = sz1 - 1;
        }
        // string outputs: their string counts follow (decode_frameheader.c:217-236)
        h.nbStrings.assign(nbOut, 0);
        for (size_t n = 0; n < nbOut; n++)
            if (h.types[n] == TY_STRING && !rd.varint(h.nbStrings[n])) { err = "truncated frame header"; return E_SRC_SMALL; }
        if (version >= 22 && hasComment) {
            uint64_t c;
            if (!rd.varint(c) || c == 0 || c > size_t(rd.end - rd.p)) { err = "bad comment"; return E_CORRUPT; }
            rd.p += c;
        }
        h.end = size_t(rd.p - src);
        if (h.hasCompressedCk) {
            if (h.end + 1 > size) { err = "truncated header"; return E_SRC_SMALL; }
            h.hdrCk = true;
            h.end++;
        }
    }
    h.outType = h.types[0];
    h.outSize = h.sizes[0];
    return 0;
}

uint64_t frameOutputLayout(const FrameHeader& h, std::vector<uint64_t>& offsets, std::vector<uint64_t>* lensOffsets)
{
    offsets.resize(h.sizes.size());
    if (lensOffsets) lensOffsets->assign(h.sizes.size(), 0);
    uint64_t extent = 0;
    for (size_t o = 0; o < h.sizes.size(); o++) {
        offsets[o] = (extent + 15) & ~uint64_t(15);
        extent = offsets[o] + h.sizes[o];
        if (h.types[o] == TY_STRING) {
            uint64_t const lo = (extent + 15) & ~uint64_t(15);
            if (lensOffsets) (*lensOffsets)[o] = lo;
            extent = lo + 4 * h.nbStrings[o];
        }
    }
    return extent;
}

int DecodePlan::planFrame(int f, const uint8_t* src, size_t size, size_t dstCap, bool ckContent,
                          bool ckCompressed, std::string& err)
{
    FrameHeader h;
    int rc = parseFrameHeader(src, size, h, err);
    if (rc) return rc;
    FramePlan& fp = frames[f];
    size_t const nbOut = h.sizes.size();
    uint64_t const extent = frameOutputLayout(h, fp.outOffs, &fp.lensOffs);
    fp.nbStrings = h.nbStrings;
    fp.stringsDone.assign(nbOut, 0);
    fp.outSizes = h.sizes;
    fp.outTypes = h.types;
    fp.outWidths.assign(nbOut, 0);
    if (extent > dstCap) { err = "destination too small"; return E_DST_SMALL; }
    size_t pos = h.end;
    // header checksum byte: low 8 bits of XXH3 over the header; verified on
    // the device together with the block checksums.
    if (h.hdrCk && ckCompressed)
        hashes.push_back(PlanHash{ f, HW_FRAME, 0, pos - 1, src[pos - 1], E_CK_COMPRESSED, true });
    fp.outType = h.outType;
    std::vector<uint64_t> produced(nbOut, 0);
    for (;;) {
        // versions before 21 hold one block and no end-of-frame marker
        // (decompress2.c:1689-1714)
        if (h.version >= 21) {
            if (pos >= size) { err = "missing end-of-frame marker"; return E_SRC_SMALL; }
            if (src[pos] == 0) { pos++; break; }
        }
        size_t consumed = 0;
        rc = planBlock(f, h.version, src, size, pos, &consumed, h.hasContentCk, h.hasCompressedCk, ckContent,
                       ckCompressed, produced, err);
        if (rc) return rc;
        pos += consumed;
        if (h.version < 21) break;
    }
    for (size_t o = 0; o < nbOut; o++) {
        if (produced[o] != h.sizes[o]) { err = "decoded size does not match the frame header"; return E_CORRUPT; }
        if (h.types[o] == TY_STRING && fp.stringsDone[o] != h.nbStrings[o]) {
            err = "string count does not match the frame header";
            return E_CORRUPT;
        }
    }
    fp.decodedSize = extent;
    fp.frameBytes = pos;
    return 0;
}

// One block: chunk header (src/openzl/decompress/decode_frameheader.c:938-1171),
// stored streams (src/openzl/decompress/decompress2.c:632-834), checksums
// (decompress2.c:1478-1570).
int DecodePlan::planBlock(int f, unsigned version, const uint8_t* src, size_t size, size_t start,
                          size_t* consumed, bool hasContentCk, bool hasCompressedCk, bool ckContent,
                          bool ckCompressed, std::vector<uint64_t>& produced, std::string& err)
{
    FramePlan& fp = frames[f];
    size_t const nbOutputs = fp.outOffs.size();
    Reader rd{ src + start, src + size };
    uint64_t nd, ns;
    // counts: single bytes before v9, varints after; the decoder count is
    // stored +1 from v21 (decode_frameheader.c:954-972)
    if (version < 9) {
        if (rd.end - rd.p < 2) { err = "truncated block header"; return E_SRC_SMALL; }
        nd = rd.p[0];
        ns = rd.p[1];
        rd.p += 2;
    } else {
        if (!rd.varint(nd)) { err = "bad decoder count"; return E_CORRUPT; }
        if (version >= 21) {
            if (nd == 0) { err = "bad decoder count"; return E_CORRUPT; }
            nd--;
        }
        if (!rd.varint(ns)) { err = "bad stored-stream count"; return E_CORRUPT; }
    }
    // ZL_runtimeNodeLimit / ZL_runtimeStreamLimit (src/openzl/common/limits.c:18-46)
    uint64_t const nodeLimit = version < 9 ? 256 : version < 20 ? 10000 : 20000;
    uint64_t const streamLimit = version < 9 ? 256 : version < 16 ? 10000 : 110000;
    if (nd >= nodeLimit || ns >= streamLimit) { err = "graph too large"; return E_LIMIT; }
    if (nd + ns < nbOutputs) { err = "fewer streams than outputs"; return E_CORRUPT; }
    // before v21 the checksum flags open the block header (decode_frameheader.c:1002-1011)
    if (version < 21) {
        if (rd.p >= rd.end) { err = "truncated block header"; return E_SRC_SMALL; }
        hasContentCk = rd.p[0] & 1;
        hasCompressedCk = (rd.p[0] >> 1) & 1;
        rd.p++;
    }
    std::vector<uint64_t> trt, ids, hflags, vflags, rflags;
    if (!rd.unpack(trt, nd, 1)) { err = "truncated codec types"; return E_SRC_SMALL; }
    for (uint64_t t : trt)
        if (t) { err = "custom codecs are not on the GPU path"; return E_TRANSFORM; }
    if (!rd.unpack(ids, nd, nextPow2Bits(T_ID_END))) { err = "truncated codec ids"; return E_SRC_SMALL; }
    if (!rd.unpack(hflags, nd, 1)) { err = "truncated header sizes"; return E_SRC_SMALL; }
    std::vector<uint64_t> hsz(nd, 0), hstart(nd, 0);
    uint64_t totalTH = 0;
    for (size_t u = 0; u < nd; u++) {
        if (hflags[u]) {
            uint64_t v;
            if (!rd.varint(v)) { err = "bad header size"; return E_CORRUPT; }
            hsz[u] = v + 1;
        }
        hstart[u] = totalTH;
        totalTH += hsz[u];
    }
    if (!rd.unpack(vflags, nd, 1)) { err = "truncated VO counts"; return E_SRC_SMALL; }
    std::vector<uint64_t> nbVO(nd, 0), nbRegen(nd, 1);
    for (size_t u = 0; u < nd; u++)
        if (vflags[u]) {
            uint64_t v;
            if (!rd.varint(v)) { err = "bad VO count"; return E_CORRUPT; }
            nbVO[u] = v + 1;
        }
    // one regenerated stream per decoder before v16 (decode_frameheader.c:1068-1082)
    if (version >= 16) {
        if (!rd.unpack(rflags, nd, 1)) { err = "truncated regen counts"; return E_SRC_SMALL; }
    } else {
        rflags.assign(nd, 0);
    }
    uint64_t totalRegen = 0;
    for (size_t u = 0; u < nd; u++) {
        if (rflags[u]) {
            uint64_t v;
            if (!rd.varint(v)) { err = "bad regen count"; return E_CORRUPT; }
            nbRegen[u] = v + 2;
        }
        totalRegen += nbRegen[u];
    }
    std::vector<uint64_t> dist;
    if (!rd.unpack(dist, totalRegen, nextPow2Bits(totalRegen + ns))) { err = "truncated distances"; return E_SRC_SMALL; }
    std::vector<uint64_t> storedSize(ns);
    for (size_t i = 0; i < ns; i++)
        if (!rd.varint(storedSize[i]) || storedSize[i] >= 0xFFFFFFFFull) { err = "bad stored size"; return E_CORRUPT; }

    // ---- stream slots -----------------------------------------------------
    size_t const total = ns + totalRegen;
    size_t const firstOutput = total - nbOutputs;
    int const sBase = int(streams.size());
    int const nBase = int(nodes.size());
    streams.resize(streams.size() + total);
    std::vector<char> isRegen(total, 0);
    std::vector<Sig> sigs(nd);
    {
        size_t sidx = 0, d = 0;
        for (size_t u = 0; u < nd; u++) {
            sigs[u] = signature(uint32_t(ids[u]));
            if (!sigs[u].known) {
                err = "codec id " + std::to_string(ids[u]) + " is not on the GPU path";
                return E_TRANSFORM;
            }
            if (!sigs[u].vo && nbVO[u]) { err = "unexpected variable inputs"; return E_CORRUPT; }
            if (nbRegen[u] != 1) { err = "multi-output decoders are not on the GPU path"; return E_TRANSFORM; }
            size_t const inEnd = sidx + size_t(sigs[u].nbSO) + nbVO[u];
            if (inEnd > firstOutput) { err = "graph inconsistency"; return E_CORRUPT; }
            size_t const o = inEnd + dist[d];
            d += nbRegen[u];
            if (o >= total || isRegen[o]) { err = "graph inconsistency"; return E_CORRUPT; }
            isRegen[o] = 1;
            sidx = inEnd;
        }
    }
    size_t pos = size_t(rd.p - src);
    size_t const thStart = pos;
    pos += totalTH;
    if (pos > size) { err = "truncated codec headers"; return E_SRC_SMALL; }
    {
        size_t st = 0;
        for (size_t i = 0; i < total; i++) {
            if (isRegen[i]) continue;
            if (st == ns) { err = "stream count mismatch"; return E_CORRUPT; }
            if (pos + storedSize[st] > size) { err = "truncated stored stream"; return E_SRC_SMALL; }
            PlanStream& s = streams[sBase + int(i)];
            s.type = TY_SERIAL;
            s.w = 1;
            s.n = storedSize[st];
            s.loc = L_FRAME;
            s.frame = f;
            s.off = pos;
            s.host = src + pos;
            pos += storedSize[st];
            st++;
        }
        if (st != ns) { err = "stream count mismatch"; return E_CORRUPT; }
    }
    uint32_t contentCk = 0;
    if (hasContentCk) {
        if (pos + 4 > size) { err = "truncated checksum"; return E_SRC_SMALL; }
        contentCk = readLE32(src + pos);
        pos += 4;
    }
    if (hasCompressedCk) {
        if (pos + 4 > size) { err = "truncated checksum"; return E_SRC_SMALL; }
        if (ckCompressed) {
            // versions before 21 hash the frame from its first byte, later
            // ones the block only (decompress2.c:1494-1500)
            size_t const hs = version < 21 ? 0 : start;
            hashes.push_back(PlanHash{ f, HW_FRAME, hs, pos - hs, readLE32(src + pos), E_CK_COMPRESSED, false });
        }
        pos += 4;
    }

    // ---- nodes and sizes (forward, decoder order) ------------------------
    auto S = [&](size_t local) -> PlanStream& { return streams[sBase + int(local)]; };
    {
        size_t sidx = 0, d = 0;
        for (size_t u = 0; u < nd; u++) {
            PlanNode nodeU;
            nodeU.id = uint32_t(ids[u]);
            nodeU.frame = f;
            nodeU.hdr = src + thStart + hstart[u];
            nodeU.hsz = size_t(hsz[u]);
            Sig const& sg = sigs[u];
            size_t const nbIn = size_t(sg.nbSO) + nbVO[u];
            nodeU.ins.resize(nbIn);
            for (size_t k = 0; k < nbIn; k++) {
                size_t const inb = nbIn - 1 - k; // decoder input order is reversed
                PlanStream& s = S(sidx + k);
                if (s.type == 0) { err = "input stream not filled"; return E_CORRUPT; }
                if (int(inb) < sg.nbSO ? s.type != sg.so[inb] : !(s.type & sg.vo)) {
                    err = "input type mismatch";
                    return E_CORRUPT;
                }
                nodeU.ins[inb] = sBase + int(sidx + k);
            }
            size_t const oLocal = sidx + nbIn + dist[d];
            d += nbRegen[u];
            nodeU.out = sBase + int(oLocal);
            PlanStream& O = S(oLocal);
            O.producer = nBase + int(u);
            O.type = sg.out;
            const uint8_t* h = nodeU.hdr;
            size_t const hs = nodeU.hsz;
            auto in = [&](int k) -> PlanStream& { return streams[nodeU.ins[k]]; };
            switch (nodeU.id) {
                case T_DELTA: {
                    O.w = in(0).w;
                    if (hs) {
                        if (hs != in(0).w) { err = "delta header size"; return E_CORRUPT; }
                        O.n = in(0).n + 1;
                    } else {
                        if (in(0).n) { err = "delta without first value"; return E_CORRUPT; }
                        O.n = 0;
                    }
                    break;
                }
                case T_ZIGZAG: O.w = in(0).w; O.n = in(0).n; break;
                case T_TSPLIT: {
                    if (nbIn == 0) { err = "empty transpose"; return E_CORRUPT; }
                    for (size_t k = 0; k < nbIn; k++)
                        if (in(int(k)).n != in(0).n || in(int(k)).w != 1) { err = "transpose plane sizes"; return E_CORRUPT; }
                    O.w = uint32_t(nbIn);
                    O.n = in(0).n;
                    break;
                }
                case T_CONV_NUM_TO_STRUCT: {
                    uint32_t w = in(0).w;
                    if (!(w == 1 || w == 2 || w == 4 || w == 8)) { err = "numeric width"; return E_CORRUPT; }
                    O.w = w; O.n = in(0).n;
                    break;
                }
                case T_CONV_STRUCT_TO_NUM: O.w = in(0).w; O.n = in(0).n; break;
                case T_CONV_SERIAL_TO_NUM:
                case T_CONV_SERIAL_TO_STRUCT: O.w = 1; O.n = in(0).n * in(0).w; break;
                case T_CONV_NUM_TO_SERIAL: {
                    if (hs != 1 || h[0] > 3) { err = "conversion header"; return E_HEADER; }
                    uint32_t w = 1u << h[0];
                    uint64_t b = in(0).bytes();
                    if (b % w) { err = "conversion size"; return E_CORRUPT; }
                    O.w = w; O.n = b / w;
                    break;
                }
                case T_CONV_STRUCT_TO_SERIAL: {
                    Reader hr{ h, h + hs };
                    uint64_t w;
                    if (!hr.varint(w) || w == 0 || hr.p != h + hs) { err = "conversion header"; return E_HEADER; }
                    uint64_t b = in(0).bytes();
                    if (b % w) { err = "conversion size"; return E_CORRUPT; }
                    O.w = uint32_t(w); O.n = b / w;
                    break;
                }
                case T_BITPACK_SERIAL:
                case T_BITPACK_INT: {
                    if (hs < 1 || hs > 2) { err = "bitpack header"; return E_HEADER; }
                    uint32_t w = 1u << ((h[0] >> 6) & 3);
                    int nbBits = 1 + (h[0] & 0x3f);
                    if (uint32_t(nbBits) > 8 * w) { err = "bitpack width"; return E_CORRUPT; }
                    if (nodeU.id == T_BITPACK_SERIAL && w != 1) { err = "bitpack width"; return E_HEADER; }
                    uint64_t srcSize = in(0).n;
                    uint64_t maxN = srcSize * 8 / uint64_t(nbBits);
                    uint64_t n = maxN;
                    if (hs > 1) {
                        if (h[1] > maxN) { err = "bitpack header"; return E_CORRUPT; }
                        n -= h[1];
                    }
                    if ((n * uint64_t(nbBits) + 7) / 8 != srcSize) { err = "bitpack size"; return E_CORRUPT; }
                    O.w = w; O.n = n;
                    nodeU.nbBits = uint8_t(nbBits);
                    break;
                }
                case T_FLATPACK: {
                    PlanStream& A = in(0);
                    PlanStream& P = in(1);
                    if (A.n > 256) { err = "flatpack alphabet"; return E_CORRUPT; }
                    uint64_t n = 0;
                    unsigned nb = A.n <= 1 ? unsigned(A.n) : 1u + unsigned(highbit32(uint32_t(A.n - 1)));
                    if (P.n && A.n) {
                        if (P.loc != L_FRAME) { err = "flatpack over a regenerated stream"; return E_LIMIT; }
                        uint32_t last = src[P.off + P.n - 1] | 1u;
                        uint64_t pad = uint64_t(__builtin_clz(last << 24)) + 1;
                        n = (8 * P.n - pad) / nb;
                    }
                    O.w = 1; O.n = n;
                    nodeU.nbBits = uint8_t(nb);
                    break;
                }
                case T_FLOATDEC: {
                    if (hs != 1 || h[0] > 2) { err = "float header"; return E_CORRUPT; }
                    uint32_t const sfw = h[0] == 0 ? 3 : (h[0] == 1 ? 1 : 2);
                    if (in(0).n != in(1).n || in(0).w != sfw || in(1).w != 1) { err = "float inputs"; return E_CORRUPT; }
                    O.w = h[0] == 0 ? 4 : 2;
                    O.n = in(1).n;
                    break;
                }
                case T_SEP_STRING: { // DI_revert_VSF_separation (decode_conversion_binding.c:230-275)
                    PlanStream& L = in(1);
                    if (!(L.w == 1 || L.w == 2 || L.w == 4 || L.w == 8)) { err = "string lengths width"; return E_CORRUPT; }
                    O.w = 1;
                    O.n = in(0).bytes();
                    O.lens = nodeU.ins[1];
                    if (L.host) { // lengths known here: their sum must be the content size
                        uint64_t sum = 0;
                        for (uint64_t i = 0; i < L.n; i++) {
                            uint64_t v = 0;
                            for (uint32_t b = 0; b < L.w; b++) v |= uint64_t(L.host[i * L.w + b]) << (8 * b);
                            if (v > 0xffffffffull) { err = "string length above 32 bits"; return E_CORRUPT; }
                            sum += v;
                        }
                        if (sum != O.n) { err = "string lengths do not add up to the content"; return E_CORRUPT; }
                    }
                    break;
                }
                case T_TOKENIZE_FIXED:
                case T_TOKENIZE_NUMERIC: {
                    uint32_t iw = in(1).w;
                    if (!(iw == 1 || iw == 2 || iw == 4 || iw == 8)) { err = "index width"; return E_CORRUPT; }
                    O.w = in(0).w; O.n = in(1).n;
                    break;
                }
                case T_SPLITN:
                case T_SPLITN_STRUCT:
                case T_SPLITN_NUM: {
                    uint32_t w = 1;
                    if (nbIn == 0) {
                        if (hs) {
                            Reader hr{ h, h + hs };
                            uint64_t v;
                            if (!hr.varint(v)) { err = "splitN header"; return E_CORRUPT; }
                            w = uint32_t(v);
                        }
                    } else {
                        w = in(0).w;
                    }
                    uint64_t n = 0;
                    for (size_t k = 0; k < nbIn; k++) {
                        if (in(int(k)).w != w || in(int(k)).type != in(0).type) { err = "splitN inputs"; return E_CORRUPT; }
                        n += in(int(k)).n;
                    }
                    O.w = w; O.n = n;
                    break;
                }
                case T_CONST_SERIAL:
                case T_CONST_FIXED: {
                    if (in(0).n != 1) { err = "constant input"; return E_CORRUPT; }
                    Reader hr{ h, h + hs };
                    uint64_t n;
                    if (!hr.varint(n) || hr.p != h + hs || n < 1) { err = "constant header"; return E_CORRUPT; }
                    O.w = in(0).w; O.n = n;
                    break;
                }
                case T_NCOUNT: {
                    PlanStream& I = in(0);
                    if (I.loc != L_FRAME) { err = "ncount over a regenerated stream"; return E_LIMIT; }
                    int16_t norm[256];
                    unsigned nbSym = 0;
                    long r = parseNCount(norm, nbSym, src + I.off, size_t(I.n));
                    if (r < 0 || uint64_t(r) != I.n) { err = "bad normalized counts"; return E_CORRUPT; }
                    size_t const off = (params.size() + 15) & ~size_t(15);
                    params.resize(off + 2 * nbSym);
                    std::memcpy(params.data() + off, norm, 2 * nbSym);
                    O.w = 2; O.n = nbSym;
                    O.loc = L_PARAM;
                    O.off = off;
                    nodeU.dead = true; // executed here, on the host
                    break;
                }
                case T_FSE: {
                    PlanStream& N = in(0);
                    if (N.w != 2) { err = "FSE counts width"; return E_CORRUPT; }
                    if (N.n < 2 || N.n > 256) { err = "FSE symbol count"; return E_CORRUPT; }
                    // The counts are host-known: decoded from an ncount header
                    // here, or stored raw in the frame (small alphabets).
                    if (N.loc == L_PARAM) {
                        nodeU.paramOff = N.off;
                    } else if (N.host) {
                        size_t const off = (params.size() + 15) & ~size_t(15);
                        params.resize(off + 2 * N.n);
                        std::memcpy(params.data() + off, N.host, 2 * N.n);
                        nodeU.paramOff = off;
                    } else {
                        err = "FSE counts regenerated on the device";
                        return E_LIMIT;
                    }
                    int16_t normBuf[256];
                    std::memcpy(normBuf, params.data() + nodeU.paramOff, 2 * N.n);
                    const int16_t* norm = normBuf;
                    unsigned sum = 0;
                    for (uint64_t i = 0; i < N.n; i++) {
                        if (norm[i] < -1) { err = "FSE counts"; return E_CORRUPT; }
                        sum += norm[i] == -1 ? 1u : unsigned(norm[i]);
                    }
                    if (sum == 0 || (sum & (sum - 1))) { err = "FSE counts sum"; return E_CORRUPT; }
                    int tl = highbit32(sum);
                    if (tl < 5 || tl > 12) { err = "FSE table log"; return E_CORRUPT; }
                    if (hs < 2 || hs > 9 || (h[0] != 2 && h[0] != 4)) { err = "FSE header"; return E_CORRUPT; }
                    uint64_t dstSize = readLEn(h + 1, hs - 1);
                    if (dstSize < 2 || dstSize >= (1ull << 32)) { err = "FSE size"; return E_CORRUPT; }
                    if (in(1).n >= (1ull << 32)) { err = "FSE stream size"; return E_LIMIT; }
                    O.w = 1; O.n = dstSize;
                    nodeU.nbBits = uint8_t(tl);
                    break;
                }
                case T_HUF: {
                    if (in(0).w != 1) { err = "Huffman weights width"; return E_CORRUPT; }
                    if (in(0).n < 2 || in(0).n > 256) { err = "Huffman weights count"; return E_CORRUPT; }
                    if (hs < 2 || hs > 9) { err = "Huffman header"; return E_CORRUPT; }
                    uint64_t dstSize = readLEn(h + 1, hs - 1);
                    if (dstSize < 2 || dstSize >= (1ull << 32)) { err = "Huffman size"; return E_CORRUPT; }
                    if (in(1).n >= (1ull << 32)) { err = "Huffman stream size"; return E_LIMIT; }
                    O.w = 1; O.n = dstSize;
                    break;
                }
                case T_HUF16: {
                    // decode_entropy_binding.c:415-467, decode_huffman_kernel.c:196-290
                    if (in(0).w != 1) { err = "Huffman weights width"; return E_CORRUPT; }
                    if (in(0).n < 2 || in(0).n > 65536) { err = "Huffman weights count"; return E_CORRUPT; }
                    if (hs < 2 || hs > 9) { err = "Huffman header"; return E_CORRUPT; }
                    uint64_t dstSize = readLEn(h + 1, hs - 1);
                    if (dstSize < 2 || dstSize >= (1ull << 32)) { err = "Huffman size"; return E_CORRUPT; }
                    PlanStream& I = in(1);
                    if (I.loc != L_FRAME) { err = "16-bit Huffman over a regenerated bitstream"; return E_LIMIT; }
                    // the stream table: symbol count and byte size (LE32) before each stream
                    uint32_t const nbStreams = (h[0] & 1) ? 4u : 1u;
                    uint32_t tab[16] = { 0 };
                    uint64_t pos = 0, done = 0;
                    const uint8_t* const b = src + I.off;
                    for (uint32_t k = 0; k < nbStreams; k++) {
                        if (pos + 8 > I.n) { err = "Huffman stream table"; return E_CORRUPT; }
                        uint32_t const cnt = uint32_t(readLEn(b + pos, 4)), sz = uint32_t(readLEn(b + pos + 4, 4));
                        pos += 8;
                        if (pos + sz > I.n || done + cnt > dstSize || sz == 0) { err = "Huffman stream table"; return E_CORRUPT; }
                        tab[k] = uint32_t(pos);
                        tab[4 + k] = sz;
                        tab[8 + k] = cnt;
                        tab[12 + k] = uint32_t(done);
                        pos += sz;
                        done += cnt;
                    }
                    if (pos != I.n || done != dstSize) { err = "Huffman stream table"; return E_CORRUPT; }
                    size_t const off = (params.size() + 15) & ~size_t(15);
                    params.resize(off + sizeof(tab));
                    std::memcpy(params.data() + off, tab, sizeof(tab));
                    nodeU.paramOff = off;
                    nodeU.nbBits = uint8_t(nbStreams);
                    O.w = 2; O.n = dstSize;
                    break;
                }
                default:
                    err = "unsupported codec";
                    return E_TRANSFORM;
            }
            if (sg.view && in(0).host) O.host = in(0).host;
            nodes.push_back(std::move(nodeU));
            sidx += nbIn;
        }
    }

    // ---- outputs: the last stream slots, output o in slot total - 1 - o --
    std::vector<uint64_t> const before = produced;
    std::vector<uint64_t> const stringsBefore = fp.stringsDone;
    for (size_t o = 0; o < nbOutputs; o++) {
        PlanStream& OUT = S(total - 1 - o);
        if (OUT.type == 0) { err = "output not regenerated"; return E_CORRUPT; }
        if (OUT.type == TY_STRING) {
            // the string node's inputs are written straight into the output
            // (content) and after it (lengths); the node itself runs no kernel
            if (OUT.producer < 0 || nodes[OUT.producer].id != T_SEP_STRING) {
                err = "string outputs come from separate_string_components only";
                return E_TRANSFORM;
            }
            PlanNode& sn = nodes[OUT.producer];
            sn.dead = true;
            PlanStream& L = streams[sn.ins[1]];
            if (fp.stringsDone[o] + L.n > fp.nbStrings[o]) { err = "more strings than the frame header says"; return E_CORRUPT; }
            fp.stringsDone[o] += L.n;
        }
        if (fp.outWidths[o] == 0) {
            fp.outWidths[o] = OUT.w;
            fp.outTypes[o] = OUT.type;
        } else if (fp.outWidths[o] != OUT.w || fp.outTypes[o] != OUT.type) {
            err = "output type changes between blocks";
            return E_CORRUPT;
        }
        if (produced[o] + OUT.bytes() > fp.outSizes[o]) { err = "output larger than the frame header says"; return E_CORRUPT; }
        if (OUT.producer < 0 && OUT.bytes()) {
            // the frame stores the output verbatim: copy it into place
            directCopies.push_back(PlanCopy{ f, OUT.off, fp.outOffs[o] + produced[o], OUT.bytes() });
        }
        produced[o] += OUT.bytes();
    }
    fp.outWidth = fp.outWidths[0];
    fp.outType = fp.outTypes[0];

    // ---- fusion of numeric chains (delta <- zigzag <- view <- tsplit|bitpack)
    auto isNumView = [&](const PlanNode& nd_) {
        return !nd_.dead && signature(nd_.id).view;
    };
    // consumers before producers, so the outermost node absorbs the whole chain
    for (int u = int(nodes.size()) - 1; u >= nBase; u--) {
        PlanNode& C = nodes[u];
        if (C.dead) continue;
        if (C.id != T_DELTA && C.id != T_ZIGZAG && C.id != T_TSPLIT && C.id != T_BITPACK_INT
            && C.id != T_BITPACK_SERIAL)
            continue;
        uint32_t const w = streams[C.out].w;
        if (C.id == T_TSPLIT) {
            if (w == 1 || w == 2 || w == 4 || w == 8) C.srcMode = SRC_PLANES;
            continue; // general widths use the transpose kernel
        }
        if (C.id == T_BITPACK_INT || C.id == T_BITPACK_SERIAL) {
            C.srcMode = SRC_BITPACK;
            continue;
        }
        int cur = C.ins[0];
        if (C.id == T_DELTA) {
            C.delta = 1;
            int p = streams[cur].producer;
            if (p >= 0 && !nodes[p].dead && nodes[p].id == T_ZIGZAG) {
                C.zigzag = 1;
                nodes[p].dead = true;
                cur = nodes[p].ins[0];
            }
        } else {
            C.zigzag = 1;
        }
        int p = streams[cur].producer;
        std::vector<int> views;
        while (p >= 0 && isNumView(nodes[p])) {
            views.push_back(p);
            cur = nodes[p].ins[0];
            p = streams[cur].producer;
        }
        if (p >= 0 && !nodes[p].dead && nodes[p].id == T_TSPLIT && nodes[p].ins.size() == w) {
            C.srcMode = SRC_PLANES;
            C.ins = nodes[p].ins;
            nodes[p].dead = true;
            for (int v : views) nodes[v].dead = true;
        } else if (p >= 0 && !nodes[p].dead && (nodes[p].id == T_BITPACK_INT || nodes[p].id == T_BITPACK_SERIAL)
                   && streams[nodes[p].out].w == w) {
            C.srcMode = SRC_BITPACK;
            C.nbBits = nodes[p].nbBits;
            C.ins = nodes[p].ins;
            nodes[p].dead = true;
            for (int v : views) nodes[v].dead = true;
        } else {
            C.srcMode = SRC_PLAIN;
            if (!views.empty()) {
                // read through the views directly
                C.ins = { cur };
                for (int v : views) nodes[v].dead = true;
            }
        }
    }

    // ---- placement (reverse decoder order) ------------------------------
    for (size_t o = 0; o < nbOutputs; o++) {
        PlanStream& OUT = S(total - 1 - o);
        OUT.loc = L_OUT;
        OUT.frame = f;
        OUT.off = fp.outOffs[o] + before[o];
        if (OUT.type != TY_STRING) continue;
        const PlanNode& sn = nodes[OUT.producer];
        uint64_t const at[2] = { OUT.off, fp.lensOffs[o] + 4 * stringsBefore[o] };
        for (int k = 0; k < 2; k++) {
            PlanStream& I = streams[sn.ins[k]];
            if (k == 1 && I.w != 4) { // narrower lengths: widened into place
                widens.push_back(PlanWiden{ sn.ins[1], f, at[1] });
                continue;
            }
            if (I.producer < 0) { // stored: copied into place
                if (I.bytes()) directCopies.push_back(PlanCopy{ f, I.off, at[k], I.bytes() });
            } else {
                I.loc = L_OUT;
                I.frame = f;
                I.off = at[k];
            }
        }
    }
    auto alloc = [&](PlanStream& s) {
        s.loc = L_ARENA;
        s.off = arenaBytes;
        arenaBytes += (s.bytes() + 63) & ~uint64_t(63);
    };
    for (int u = int(nodes.size()) - 1; u >= nBase; u--) {
        PlanNode& nd_ = nodes[u];
        if (nd_.dead) continue;
        Sig const sg = signature(nd_.id);
        PlanStream& O = streams[nd_.out];
        if (sg.view) {
            PlanStream& I = streams[nd_.ins[0]];
            if (O.loc == L_NONE) {
                O.loc = L_ALIAS;
                O.parent = nd_.ins[0];
            } else if (I.loc == L_NONE && I.producer >= 0) {
                I.loc = L_SUB;
                I.parent = nd_.out;
                I.off = 0;
            }
            // else: stored input into a placed output -> copy task (emitted later)
            continue;
        }
        if (O.loc == L_NONE) alloc(O);
        if (sg.concat) {
            uint64_t off = 0;
            for (int s : nd_.ins) {
                PlanStream& I = streams[s];
                if (I.loc == L_NONE && I.producer >= 0) {
                    I.loc = L_SUB;
                    I.parent = nd_.out;
                    I.off = off;
                }
                off += I.bytes();
            }
        }
    }
    *consumed = pos - start;
    // content checksum: XXH3 of the block's outputs one after another
    // (STREAM_hashLastCommit_xxh3low32, src/openzl/common/stream.c:727-773)
    // (a string output contributes its content, then from v15 its 4-byte
    // lengths, stream.c:757-766)
    if (hasContentCk && ckContent) {
        bool const strings = [&] {
            for (int t : fp.outTypes) if (t == TY_STRING) return true;
            return false;
        }();
        if (nbOutputs == 1 && !strings) {
            hashes.push_back(PlanHash{ f, HW_OUTPUT, fp.outOffs[0] + before[0], produced[0] - before[0], contentCk, 14, false });
        } else {
            std::vector<PlanGather> segs;
            uint64_t const base = arenaBytes;
            uint64_t at = base;
            for (size_t o = 0; o < nbOutputs; o++) {
                uint64_t const b = produced[o] - before[o];
                if (b) segs.push_back(PlanGather{ f, fp.outOffs[o] + before[o], at, b });
                at += b;
                if (fp.outTypes[o] == TY_STRING && version >= 15) {
                    uint64_t const lb = 4 * (fp.stringsDone[o] - stringsBefore[o]);
                    if (lb) segs.push_back(PlanGather{ f, fp.lensOffs[o] + 4 * stringsBefore[o], at, lb });
                    at += lb;
                }
            }
            arenaBytes += (at - base + 63) & ~uint64_t(63);
            gathers.insert(gathers.end(), segs.begin(), segs.end());
            hashes.push_back(PlanHash{ f, HW_ARENA, base, at - base, contentCk, 14, false });
        }
    }
    return 0;
}

} // namespace ozl

// ---------------------------------------------------------------------------
// Layout: dependency levels, copy tasks, per-(level, kind) task arrays with
// absolute device addresses. Called once with null bases to size the pools,
// then again with the real allocations.
namespace ozl {

namespace {

struct Pool {
    std::vector<uint8_t> bytes;
    template <class T>
    size_t put(const std::vector<T>& v)
    {
        size_t off = (bytes.size() + 63) & ~size_t(63);
        bytes.resize(off + v.size() * sizeof(T));
        if (!v.empty()) std::memcpy(bytes.data() + off, v.data(), v.size() * sizeof(T));
        return off;
    }
};

struct Buckets {
    std::vector<NumPipeTask> num;
    std::vector<TransposeTask> tr;
    std::vector<CopyTask> copy;
    std::vector<ConstTask> cst;
    std::vector<FseTask> fse;
    std::vector<HufTask> huf;
    std::vector<Huf16Task> huf16;
    std::vector<TokenizeTask> tok;
    std::vector<WidenTask> widen;
    std::vector<FloatDecTask> flt;
    std::vector<FlatpackTask> flat;
};

uint32_t ceilDiv(uint64_t a, uint64_t b) { return uint32_t((a + b - 1) / b); }

// Algorithmic bytes of one task: what it must read plus what it must write.
uint64_t taskBytes(const CopyTask& t) { return 2 * t.bytes; }
uint64_t taskBytes(const ConstTask& t) { return t.n * t.w + t.w; }
uint64_t taskBytes(const FseTask& t) { return uint64_t(t.bitsSize) + t.dstSize + 2ull * t.nbSym; }
uint64_t taskBytes(const HufTask& t) { return uint64_t(t.bitsSize) + t.dstSize + t.nbWeights; }
uint64_t taskBytes(const Huf16Task& t)
{
    uint64_t b = t.nbWeights;
    for (uint32_t k = 0; k < t.nbStreams; k++) b += uint64_t(t.streamSize[k]) + 2ull * t.count[k];
    return b;
}
uint64_t taskBytes(const FlatpackTask& t) { return t.n + (t.n * t.nbBits + 7) / 8 + t.alphabetSize; }
uint64_t taskBytes(const TokenizeTask& t) { return t.n * (t.w + t.iw) + uint64_t(t.alphabetSize) * t.w; }
uint64_t taskBytes(const WidenTask& t) { return t.n * (t.w + 4); }
uint64_t taskBytes(const FloatDecTask& t) { return t.n * (t.eltType == 0 ? 8 : 4); }
uint64_t taskBytes(const TransposeTask& t) { return 2 * t.n * t.W; }
uint64_t taskBytes(const NumPipeTask& t)
{
    uint64_t const ns = t.delta ? (t.n ? t.n - 1 : 0) : t.n;
    uint64_t const src = t.srcMode == SRC_BITPACK ? (ns * t.nbBits + 7) / 8 : ns * t.w;
    return src + t.n * t.w;
}

} // namespace

int layoutPlan(const DecodePlan& plan, const uint8_t* const* dFrames, uint8_t* const* dOuts,
               uint8_t* dArena, uint8_t* dParams, uint8_t* dScratch, uint8_t* dPool,
               DeviceLayout& out, std::string& err, const std::vector<char>* frameMask)
{
    auto inPart = [&](int frame) { return !frameMask || (frame >= 0 && (*frameMask)[size_t(frame)]); };
    const auto& streams = plan.streams;
    const auto& nodes = plan.nodes;
    std::vector<uint8_t*> addrMemo(streams.size(), nullptr);
    std::vector<char> addrDone(streams.size(), 0);
    // Resolves a stream's device address (recursion depth is bounded by the
    // placement chain length, which is at most the graph depth).
    std::function<uint8_t*(int)> addr = [&](int s) -> uint8_t* {
        if (addrDone[s]) return addrMemo[s];
        const PlanStream& S = streams[s];
        uint8_t* a = nullptr;
        switch (S.loc) {
            case L_FRAME: a = const_cast<uint8_t*>(dFrames[S.frame]) + S.off; break;
            case L_OUT: a = dOuts[S.frame] + S.off; break;
            case L_ARENA: a = dArena + S.off; break;
            case L_PARAM: a = dParams + S.off; break;
            case L_SUB: a = addr(S.parent) + S.off; break;
            case L_ALIAS: a = addr(S.parent); break;
            default: a = nullptr;
        }
        addrMemo[s] = a;
        addrDone[s] = 1;
        return a;
    };

    // every input of a live decoder must have a location by now
    for (const PlanNode& nd : nodes) {
        if (nd.dead || !inPart(nd.frame)) continue;
        for (int s : nd.ins)
            if (streams[s].loc == L_NONE) {
                err = "planner: stream without a location (codec " + std::to_string(nd.id) + ")";
                return 80;
            }
    }

    // ---- levels ------------------------------------------------------------
    std::vector<int> level(nodes.size(), 0);
    auto streamLevel = [&](int s) {
        int p = streams[s].producer;
        return (p >= 0 && !nodes[p].dead) ? level[p] : 0;
    };
    struct CopyReq { int src, dst; uint64_t dstOff; int level; int frame; };
    std::vector<CopyReq> copies;
    int maxLevel = 0;
    for (size_t u = 0; u < nodes.size(); u++) {
        const PlanNode& nd = nodes[u];
        if (nd.dead) continue;
        int lv = 0;
        const PlanStream& O = streams[nd.out];
        bool const isView = nd.id == 5 || nd.id == 6 || nd.id == 7 || nd.id == 8 || nd.id == 9 || nd.id == 10;
        bool const isConcat = nd.id == 40 || nd.id == 47 || nd.id == 48;
        if (isView) {
            int const I = nd.ins[0];
            const PlanStream& IS = streams[I];
            if (O.loc == L_ALIAS || (IS.loc == L_SUB && IS.parent == nd.out)) {
                lv = streamLevel(I);
            } else {
                lv = streamLevel(I) + 1;
                copies.push_back(CopyReq{ I, nd.out, 0, lv, nd.frame });
            }
        } else if (isConcat) {
            uint64_t off = 0;
            for (int I : nd.ins) {
                const PlanStream& IS = streams[I];
                if (IS.loc == L_SUB && IS.parent == nd.out) {
                    lv = std::max(lv, streamLevel(I));
                } else {
                    int const cl = streamLevel(I) + 1;
                    copies.push_back(CopyReq{ I, nd.out, off, cl, nd.frame });
                    lv = std::max(lv, cl);
                }
                off += IS.bytes();
            }
        } else {
            for (int I : nd.ins) lv = std::max(lv, streamLevel(I));
            lv += 1;
        }
        level[u] = lv;
        maxLevel = std::max(maxLevel, lv);
    }
    if (!plan.directCopies.empty()) maxLevel = std::max(maxLevel, 1);
    std::vector<int> widenLevel;
    for (const PlanWiden& wd : plan.widens) {
        widenLevel.push_back(streamLevel(wd.stream) + 1);
        if (inPart(wd.frame)) maxLevel = std::max(maxLevel, widenLevel.back());
    }
    // multi-output blocks gather their outputs for the content checksum after
    // everything that writes them
    bool anyGather = false;
    for (const PlanGather& g : plan.gathers) anyGather |= inPart(g.frame);
    int const gatherLevel = maxLevel + 1;
    if (anyGather) maxLevel = gatherLevel;
    int const hashLevel = maxLevel + 1;

    // ---- tasks per level ---------------------------------------------------
    std::vector<Buckets> B(size_t(hashLevel) + 1);
    for (const CopyReq& c : copies) {
        if (!inPart(c.frame)) continue;
        uint64_t bytes = streams[c.src].bytes();
        if (!bytes) continue;
        CopyTask t{ addr(c.dst) + c.dstOff, addr(c.src), bytes, 0 };
        B[c.level].copy.push_back(t);
    }
    for (const PlanCopy& c : plan.directCopies) {
        if (!inPart(c.frame)) continue;
        CopyTask t{ dOuts[c.frame] + c.outOff, dFrames[c.frame] + c.frameOff, c.bytes, 0 };
        B[1].copy.push_back(t);
    }
    for (size_t k = 0; k < plan.widens.size(); k++) {
        const PlanWiden& wd = plan.widens[k];
        if (!inPart(wd.frame) || !streams[wd.stream].n) continue;
        B[widenLevel[k]].widen.push_back(WidenTask{ addr(wd.stream), reinterpret_cast<uint32_t*>(dOuts[wd.frame] + wd.outOff),
                                                    streams[wd.stream].n, streams[wd.stream].w, 0 });
    }
    for (const PlanGather& g : plan.gathers) {
        if (!inPart(g.frame)) continue;
        CopyTask t{ dArena + g.arenaOff, dOuts[g.frame] + g.outOff, g.bytes, 0 };
        B[gatherLevel].copy.push_back(t);
    }
    // pointer arrays (planes) live in the pool; collect them first
    std::vector<const uint8_t*> ptrs;
    std::vector<std::pair<size_t, size_t>> ptrFix; // (bucket task index marker) unused
    struct PendingPlanes { int lvl; bool isNum; size_t taskIdx; size_t ptrOff; };
    std::vector<PendingPlanes> pend;
    for (size_t u = 0; u < nodes.size(); u++) {
        const PlanNode& nd = nodes[u];
        if (nd.dead || !inPart(nd.frame)) continue;
        int const lv = level[u];
        const PlanStream& O = streams[nd.out];
        uint8_t* o = addr(nd.out);
        auto in = [&](int k) { return addr(nd.ins[k]); };
        switch (nd.id) {
            case 1: case 3: case 4: case 27: case 28: {
                if (nd.id == 4 && nd.srcMode != SRC_PLANES) {
                    TransposeTask t{ o, nullptr, O.n, O.w, 0 };
                    pend.push_back(PendingPlanes{ lv, false, B[lv].tr.size(), ptrs.size() });
                    for (int s : nd.ins) ptrs.push_back(addr(s));
                    B[lv].tr.push_back(t);
                    break;
                }
                NumPipeTask t{};
                t.out = o;
                t.n = O.n;
                t.w = O.w;
                t.srcMode = nd.srcMode;
                t.nbBits = nd.nbBits;
                t.zigzag = nd.zigzag;
                t.delta = nd.delta;
                if (nd.delta && O.n) {
                    uint64_t first = 0;
                    for (size_t b = 0; b < nd.hsz; b++) first |= uint64_t(nd.hdr[b]) << (8 * b);
                    t.first = first;
                }
                if (nd.srcMode == SRC_PLANES) {
                    pend.push_back(PendingPlanes{ lv, true, B[lv].num.size(), ptrs.size() });
                    for (int s : nd.ins) ptrs.push_back(addr(s));
                } else {
                    t.src = in(0);
                }
                if (O.n) B[lv].num.push_back(t);
                break;
            }
            case 5: case 6: case 7: case 8: case 9: case 10: case 40: case 47: case 48:
                break; // views and concatenations: placement or copy tasks
            case 29: {
                FlatpackTask t{ o, in(0), in(1), O.n, uint32_t(streams[nd.ins[0]].n), nd.nbBits, 0 };
                if (O.n) B[lv].flat.push_back(t);
                break;
            }
            case 33: {
                FloatDecTask t{ o, in(0), in(1), O.n, nd.hdr[0], 0 };
                if (O.n) B[lv].flt.push_back(t);
                break;
            }
            case 36: case 37: {
                TokenizeTask t{ o, in(0), in(1), O.n, uint32_t(streams[nd.ins[0]].n), streams[nd.ins[0]].w,
                                streams[nd.ins[1]].w, 0 };
                if (O.n) B[lv].tok.push_back(t);
                break;
            }
            case 44: case 45: {
                ConstTask t{ o, in(0), O.n, O.w, 0 };
                B[lv].cst.push_back(t);
                break;
            }
            case 49: {
                FseTask t{};
                t.out = o;
                t.bits = in(1);
                t.norm = reinterpret_cast<const int16_t*>(dParams + nd.paramOff);
                t.bitsSize = uint32_t(streams[nd.ins[1]].n);
                t.dstSize = uint32_t(O.n);
                t.nbSym = uint16_t(streams[nd.ins[0]].n);
                t.nbStates = nd.hdr[0];
                t.tableLog = nd.nbBits;
                B[lv].fse.push_back(t);
                break;
            }
            case 50: {
                HufTask t{};
                t.out = o;
                t.bits = in(1);
                t.weights = in(0);
                t.bitsSize = uint32_t(streams[nd.ins[1]].n);
                t.dstSize = uint32_t(O.n);
                t.nbWeights = uint16_t(streams[nd.ins[0]].n);
                t.x4 = nd.hdr[0] & 1;
                B[lv].huf.push_back(t);
                break;
            }
            case 51: {
                Huf16Task t{};
                t.out = o;
                t.weights = in(0);
                t.nbWeights = uint32_t(streams[nd.ins[0]].n);
                uint32_t tab[16];
                std::memcpy(tab, plan.params.data() + nd.paramOff, sizeof(tab));
                t.nbStreams = nd.nbBits;
                for (uint32_t k = 0; k < t.nbStreams; k++) {
                    t.stream[k] = in(1) + tab[k];
                    t.streamSize[k] = tab[4 + k];
                    t.count[k] = tab[8 + k];
                    t.dstOff[k] = tab[12 + k];
                }
                B[lv].huf16.push_back(t);
                break;
            }
            default:
                err = "layout: unexpected codec " + std::to_string(nd.id);
                return 32;
        }
    }

    // ---- pool assembly -----------------------------------------------------
    Pool pool;
    size_t const ptrOff = pool.put(ptrs);
    for (const PendingPlanes& p : pend) {
        auto* arr = reinterpret_cast<const uint8_t* const*>(dPool + ptrOff) + p.ptrOff;
        if (p.isNum) B[p.lvl].num[p.taskIdx].planes = arr;
        else B[p.lvl].tr[p.taskIdx].planes = arr;
    }
    out.launches.clear();
    uint64_t scratch = 0;
    // ---- checksums: block sums first in the scratch. A content checksum of
    // an output that one numeric-pipeline task writes whole, from its first
    // byte, gets its block sums from that task's output pass; the hash
    // launch's phase 1 covers the other checksums' blocks only.
    struct HashPlace { size_t hash; uint64_t sumsOff; uint32_t nbBlocks; bool fused; };
    std::vector<HashPlace> hp;
    for (size_t k = 0; k < plan.hashes.size(); k++) {
        const PlanHash& h = plan.hashes[k];
        if (!inPart(h.frame)) continue;
        uint32_t const nb = h.len > 240 ? uint32_t((h.len - 1) / kHashBlock) : 0;
        hp.push_back(HashPlace{ k, scratch, nb, false });
        scratch += (uint64_t(nb) * 64 + 255) & ~uint64_t(255);
    }
    {
        std::unordered_map<const uint8_t*, NumPipeTask*> numByOut;
        for (Buckets& b : B)
            for (NumPipeTask& t : b.num) numByOut.emplace(t.out, &t);
        for (HashPlace& p : hp) {
            const PlanHash& h = plan.hashes[p.hash];
            if (h.where != HW_OUTPUT || !p.nbBlocks) continue;
            auto it = numByOut.find(dOuts[h.frame] + h.off);
            if (it == numByOut.end()) continue;
            NumPipeTask& t = *it->second;
            if (t.blockSums || t.n * t.w < uint64_t(p.nbBlocks) * kHashBlock) continue;
            t.blockSums = reinterpret_cast<uint64_t*>(dScratch + p.sumsOff);
            t.hashBlocks = p.nbBlocks;
            p.fused = true;
        }
    }
    auto addTiled = [&](int kind, int lv, auto& tasks, auto tilesOf) {
        if (tasks.empty()) return;
        std::vector<TileRef> tiles;
        for (size_t i = 0; i < tasks.size(); i++) {
            uint32_t nt = tilesOf(tasks[i]);
            tasks[i].tileBase = uint32_t(tiles.size());
            for (uint32_t k = 0; k < nt; k++) tiles.push_back(TileRef{ uint32_t(i), k });
        }
        Launch L{};
        L.kind = kind;
        L.level = lv;
        for (auto& t : tasks) L.algoBytes += taskBytes(t);
        L.taskOff = pool.put(tasks);
        L.nbTasks = uint32_t(tasks.size());
        L.tileOff = pool.put(tiles);
        L.nbTiles = uint32_t(tiles.size());
        if (kind == KIND_NUMPIPE) {
            bool anyDelta = false;
            for (auto& t : tasks) anyDelta |= reinterpret_cast<const NumPipeTask&>(t).delta != 0;
            if (anyDelta) {
                L.needsScan = true;
                L.statusOff = scratch;
                L.statusBytes = 64 + 32 * uint64_t(tiles.size());
                scratch += (L.statusBytes + 255) & ~uint64_t(255);
            }
        }
        out.launches.push_back(L);
    };
    auto addPlain = [&](int kind, int lv, auto& tasks) {
        if (tasks.empty()) return;
        auto emit = [&](auto& part, uint32_t param0) {
            if (part.empty()) return;
            Launch L{};
            L.param0 = param0;
            for (auto& t : part) L.algoBytes += taskBytes(t);
            L.kind = kind;
            L.level = lv;
            L.taskOff = pool.put(part);
            L.nbTasks = uint32_t(part.size());
            out.launches.push_back(L);
        };
        if constexpr (std::is_same_v<std::decay_t<decltype(tasks[0])>, FseTask>) {
            // Two launches by table size (a lane's table takes 3 << tableLog
            // bytes of shared memory): small tables (Huffman weights and the
            // like) run many lanes per CTA. Within each, longest chunks first.
            std::vector<FseTask> small, large;
            for (auto& t : tasks) (t.tableLog <= 8 ? small : large).push_back(t);
            auto order = [](const FseTask& a, const FseTask& b) {
                return a.dstSize != b.dstSize ? a.dstSize > b.dstSize : a.tableLog > b.tableLog;
            };
            std::sort(large.begin(), large.end(), order);
            std::sort(small.begin(), small.end(), order);
            uint32_t tlLarge = 9, tlSmall = 5;
            for (auto& t : large) tlLarge = std::max<uint32_t>(tlLarge, t.tableLog);
            for (auto& t : small) tlSmall = std::max<uint32_t>(tlSmall, t.tableLog);
            emit(large, tlLarge);
            emit(small, tlSmall);
        } else {
            if constexpr (std::is_same_v<std::decay_t<decltype(tasks[0])>, HufTask>)
                std::stable_sort(tasks.begin(), tasks.end(),
                                 [](const HufTask& a, const HufTask& b) { return a.dstSize > b.dstSize; });
            emit(tasks, 0);
        }
    };
    for (int lv = 0; lv <= maxLevel; lv++) {
        Buckets& b = B[lv];
        addTiled(KIND_COPY, lv, b.copy, [](const CopyTask& t) { return ceilDiv(t.bytes, kTileBytes); });
        addTiled(KIND_CONST, lv, b.cst, [](const ConstTask& t) { return ceilDiv(t.n * t.w, kTileBytes); });
        addPlain(KIND_FSE, lv, b.fse);
        addPlain(KIND_HUF, lv, b.huf);
        for (Huf16Task& t : b.huf16) {
            t.sorted = reinterpret_cast<uint16_t*>(dScratch + scratch);
            scratch += (2ull * t.nbWeights + 255) & ~uint64_t(255);
        }
        addPlain(KIND_HUF16, lv, b.huf16);
        addTiled(KIND_FLATPACK, lv, b.flat, [](const FlatpackTask& t) { return ceilDiv(t.n, kTileBytes); });
        addTiled(KIND_TOKENIZE, lv, b.tok, [](const TokenizeTask& t) { return ceilDiv(t.n, kTileElems); });
        addTiled(KIND_WIDEN, lv, b.widen, [](const WidenTask& t) { return ceilDiv(t.n, kTileElems); });
        addTiled(KIND_FLOATDEC, lv, b.flt, [](const FloatDecTask& t) { return ceilDiv(t.n, kTileElems); });
        addTiled(KIND_TRANSPOSE, lv, b.tr, [](const TransposeTask& t) { return ceilDiv(t.n, kTileElems); });
        addTiled(KIND_NUMPIPE, lv, b.num, [](const NumPipeTask& t) { return ceilDiv(t.n, kNumTileBytes / t.w); });
    }
    // checksums: one launch after everything else
    if (!hp.empty()) {
        std::vector<HashTask> ht;
        std::vector<TileRef> blocks;
        for (const HashPlace& p : hp) {
            const PlanHash& h = plan.hashes[p.hash];
            HashTask t{};
            t.data = h.where == HW_OUTPUT ? dOuts[h.frame] + h.off
                   : h.where == HW_ARENA  ? dArena + h.off
                                          : dFrames[h.frame] + h.off;
            t.len = h.len;
            t.expected = h.expected;
            t.errCode = h.err;
            t.low8 = h.low8 ? 1 : 0;
            t.aligned8 = (reinterpret_cast<uintptr_t>(t.data) & 7) == 0;
            t.nbBlocks = p.nbBlocks;
            t.blockSums = reinterpret_cast<uint64_t*>(dScratch + p.sumsOff);
            t.blockBase = uint32_t(blocks.size());
            if (!p.fused)
                for (uint32_t k = 0; k < t.nbBlocks; k++) blocks.push_back(TileRef{ uint32_t(ht.size()), k });
            ht.push_back(t);
        }
        Launch L{};
        for (const HashTask& t : ht) L.algoBytes += t.len;
        L.kind = KIND_HASH;
        L.level = hashLevel;
        L.taskOff = pool.put(ht);
        L.nbTasks = uint32_t(ht.size());
        L.tileOff = pool.put(blocks);
        L.nbTiles = uint32_t(blocks.size());
        out.launches.push_back(L);
    }
    out.pool = std::move(pool.bytes);
    out.arenaBytes = plan.arenaBytes;
    out.scratchBytes = scratch;
    out.paramBytes = plan.params.size();
    return 0;
}

} // namespace ozl
