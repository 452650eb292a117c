// FSE table-log choice, count normalization and normalized-count header,
// shared by the host path and the device table builder (kFseTables). They
// restate src/openzl/fse/compress/fse_compress.c exactly (the tables decide
// the frame's bytes): FSE_optimalTableLog_internal (:379-396),
// FSE_normalizeM2 (:400-470), FSE_normalizeCount (:472-520) and
// FSE_writeNCount_generic (:226-338). Integer arithmetic only.
#pragma once
#include <cstddef>
#include <cstdint>

#ifdef __CUDACC__
#define OZL_HD __host__ __device__
#else
#define OZL_HD
#endif

namespace ozl {
namespace ent {

OZL_HD inline int highbit32v(uint32_t v)
{
#ifdef __CUDA_ARCH__
    return 31 - __clz(v);
#else
    return 31 - __builtin_clz(v);
#endif
}

OZL_HD inline unsigned fseTableLogOf(unsigned maxTL, uint64_t srcSize, unsigned maxSym, unsigned minus)
{
    unsigned const maxBitsSrc = unsigned(highbit32v(uint32_t(srcSize - 1))) - minus;
    unsigned const a = unsigned(highbit32v(uint32_t(srcSize))) + 1;
    unsigned const b = unsigned(highbit32v(maxSym)) + 2;
    unsigned const minBits = a < b ? a : b;
    unsigned tl = maxTL ? maxTL : 11;
    if (maxBitsSrc < tl) tl = maxBitsSrc;
    if (minBits > tl) tl = minBits;
    if (tl < 5) tl = 5;
    if (tl > 12) tl = 12;
    return tl;
}

// the second method, for distributions the first leaves unbalanced
OZL_HD inline bool fseNormalizeM2(int16_t* norm, unsigned tl, const uint32_t* count, uint64_t total, unsigned maxSym)
{
    int16_t const unassigned = -2;
    uint32_t distributed = 0;
    uint32_t const lowThreshold = uint32_t(total >> tl);
    uint32_t lowOne = uint32_t((total * 3) >> (tl + 1));
    for (unsigned s = 0; s <= maxSym; s++) {
        if (count[s] == 0) { norm[s] = 0; continue; }
        if (count[s] <= lowThreshold) { norm[s] = -1; distributed++; total -= count[s]; continue; }
        if (count[s] <= lowOne) { norm[s] = 1; distributed++; total -= count[s]; continue; }
        norm[s] = unassigned;
    }
    uint32_t toDistribute = (1u << tl) - distributed;
    if (toDistribute == 0) return true;
    if ((total / toDistribute) > lowOne) {
        lowOne = uint32_t((total * 3) / (toDistribute * 2));
        for (unsigned s = 0; s <= maxSym; s++)
            if (norm[s] == unassigned && count[s] <= lowOne) {
                norm[s] = 1;
                distributed++;
                total -= count[s];
            }
        toDistribute = (1u << tl) - distributed;
    }
    if (distributed == maxSym + 1) {
        unsigned maxV = 0, maxC = 0;
        for (unsigned s = 0; s <= maxSym; s++)
            if (count[s] > maxC) { maxV = s; maxC = count[s]; }
        norm[maxV] = int16_t(norm[maxV] + int16_t(toDistribute));
        return true;
    }
    if (total == 0) {
        for (unsigned s = 0; toDistribute > 0; s = (s + 1) % (maxSym + 1))
            if (norm[s] > 0) { toDistribute--; norm[s]++; }
        return true;
    }
    uint64_t const vStepLog = 62 - tl;
    uint64_t const mid = (uint64_t(1) << (vStepLog - 1)) - 1;
    uint64_t const rStep = ((uint64_t(1) << vStepLog) * toDistribute + mid) / uint32_t(total);
    uint64_t tmp = mid;
    for (unsigned s = 0; s <= maxSym; s++) {
        if (norm[s] != unassigned) continue;
        uint64_t const end = tmp + count[s] * rStep;
        uint32_t const w = uint32_t(end >> vStepLog) - uint32_t(tmp >> vStepLog);
        if (w < 1) return false;
        norm[s] = int16_t(w);
        tmp = end;
    }
    return true;
}

// normalized counts with low-probability symbols (-1)
OZL_HD inline bool fseNormalizeCounts(int16_t* norm, unsigned tl, const uint32_t* count, uint64_t total, unsigned maxSym)
{
    const uint32_t restToBeat[8] = { 0, 473195, 504333, 520860, 550000, 700000, 750000, 830000 };
    uint64_t const scale = 62 - tl;
    uint64_t const step = (uint64_t(1) << 62) / uint32_t(total);
    uint64_t const vStep = uint64_t(1) << (scale - 20);
    int still = 1 << tl;
    unsigned largest = 0;
    int16_t largestP = 0;
    uint32_t const lowThreshold = uint32_t(total >> tl);
    for (unsigned s = 0; s <= maxSym; s++) {
        if (count[s] == total) return true;
        if (count[s] == 0) { norm[s] = 0; continue; }
        if (count[s] <= lowThreshold) {
            norm[s] = -1;
            still--;
            continue;
        }
        int16_t p = int16_t((count[s] * step) >> scale);
        if (p < 8) p = int16_t(p + ((count[s] * step) - (uint64_t(p) << scale) > vStep * restToBeat[p]));
        if (p > largestP) { largestP = p; largest = s; }
        norm[s] = p;
        still -= p;
    }
    if (-still >= (norm[largest] >> 1)) return fseNormalizeM2(norm, tl, count, total, maxSym);
    norm[largest] = int16_t(norm[largest] + int16_t(still));
    return true;
}

// the normalized-count header; returns its size (at most 2 + 2 * 256 + 2 bytes)
OZL_HD inline size_t fseWriteNCountTo(uint8_t* out, const int16_t* norm, unsigned maxSym, unsigned tl)
{
    size_t op = 0;
    uint32_t bits = 0;
    int nb = 0;
    int remaining = (1 << tl) + 1, threshold = 1 << tl, width = int(tl) + 1;
    unsigned sym = 0;
    unsigned const alphabet = maxSym + 1;
    bool prev0 = false;
    bits |= (tl - 5) << nb;
    nb += 4;
    while (sym < alphabet && remaining > 1) {
        if (prev0) {
            unsigned start = sym;
            while (sym < alphabet && !norm[sym]) sym++;
            if (sym == alphabet) break;
            while (sym >= start + 24) {
                start += 24;
                bits += 0xFFFFu << nb;
                out[op] = uint8_t(bits);
                out[op + 1] = uint8_t(bits >> 8);
                op += 2;
                bits >>= 16;
            }
            while (sym >= start + 3) {
                start += 3;
                bits += 3u << nb;
                nb += 2;
            }
            bits += (sym - start) << nb;
            nb += 2;
            if (nb > 16) {
                out[op] = uint8_t(bits);
                out[op + 1] = uint8_t(bits >> 8);
                op += 2;
                bits >>= 16;
                nb -= 16;
            }
        }
        int count = norm[sym++];
        int const max = (2 * threshold - 1) - remaining;
        remaining -= count < 0 ? -count : count;
        count++;
        if (count >= threshold) count += max;
        bits += uint32_t(count) << nb;
        nb += width;
        nb -= (count < max);
        prev0 = (count == 1);
        while (remaining < threshold) {
            width--;
            threshold >>= 1;
        }
        if (nb > 16) {
            out[op] = uint8_t(bits);
            out[op + 1] = uint8_t(bits >> 8);
            op += 2;
            bits >>= 16;
            nb -= 16;
        }
    }
    out[op] = uint8_t(bits);
    out[op + 1] = uint8_t(bits >> 8);
    op += size_t((nb + 7) / 8);
    return op;
}

// per-symbol fields of the encoding table (fse_compress.c:160-200): bits
// read by a state of symbol s (deltaNbBits) and the offset of its states in
// the state table (deltaFindState); `cumul` is the symbol's first state slot
OZL_HD inline void fseSymbolDeltas(int c, unsigned tl, unsigned cumul, uint32_t& deltaNbBits, int32_t& deltaFindState)
{
    if (c == 0) {
        deltaNbBits = ((tl + 1) << 16) - (1u << tl);
        deltaFindState = 0;
    } else if (c == -1 || c == 1) {
        deltaNbBits = (tl << 16) - (1u << tl);
        deltaFindState = int32_t(cumul) - 1;
    } else {
        uint32_t const maxBitsOut = tl - unsigned(highbit32v(uint32_t(c) - 1));
        uint32_t const minStatePlus = uint32_t(c) << maxBitsOut;
        deltaNbBits = (maxBitsOut << 16) - minStatePlus;
        deltaFindState = int32_t(cumul) - c;
    }
}

} // namespace ent
} // namespace ozl
