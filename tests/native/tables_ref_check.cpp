// The encoder's table builders shared by host and device (fse_norm.h,
// huf_tree.h) against the reference's own functions, compiled from its
// sources into oracle/_ref/libozl_ref.so: on random histograms of many
// shapes, the FSE table log (FSE_optimalTableLog_internal), normalized counts
// (FSE_normalizeCount with low-probability counts, as
// encode_entropy_binding.c:100-106 calls it), the normalized-count header
// (FSE_writeNCount), the Huffman table log, code lengths and codes
// (HUF_buildCTable), including histograms with groups of equal counts around
// the sort's bucket cutoff, and the 16-bit-symbol Huffman table
// (ZS_largeHuffmanBuildCTable against huf16Build), and the codec decision's
// DataStats estimates (entropy bit for bit, Huffman, flat-packed and
// bit-packed sizes) are equal. Prints "bad=0" when every case agreed.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "enc_tables.h"
#include "fse_norm.h"
#include "huf_tree.h"

extern "C" {
unsigned ZS_FSE_optimalTableLog_internal(unsigned maxTableLog, size_t srcSize, unsigned maxSymbolValue, unsigned minus);
size_t ZS_FSE_normalizeCount(short* norm, unsigned tableLog, const unsigned* count, size_t srcSize,
                             unsigned maxSymbolValue, unsigned useLowProbCount);
size_t ZS_FSE_writeNCount(void* buffer, size_t bufferSize, const short* norm, unsigned maxSymbolValue,
                          unsigned tableLog);
unsigned ZS_FSE_isError(size_t code);
size_t ZS_HUF_buildCTable(size_t* CTable, const unsigned* count, unsigned maxSymbolValue, unsigned maxNbBits);
unsigned ZS_HUF_isError(size_t code);
// ZL_Report: an error code and a value, returned in two integer registers
struct RefReport {
    int code;
    size_t value;
};
struct RefHuf16CElt {
    uint16_t symbol;
    uint16_t nbBits;
};
RefReport ZS_largeHuffmanBuildCTable(RefHuf16CElt* ctable, const unsigned* histogram, uint16_t maxSymbolValue,
                                     int maxNbBits);
// DataStatsU8 (src/openzl/shared/data_stats.h) as an opaque block
double ZL_calculateEntropyU8(const unsigned* count, size_t totalElements);
void DataStatsU8_init(void* stats, const void* src, size_t srcSize);
double DataStatsU8_getEntropy(void* stats);
size_t DataStatsU8_estimateHuffmanSizeFast(void* stats, bool delta);
size_t DataStatsU8_getBitpackedSize(void* stats);
size_t DataStatsU8_getFlatpackedSize(void* stats);
size_t DataStatsU8_getCardinality(void* stats);
uint8_t DataStatsU8_getMaxElt(void* stats);
}

using namespace ozl::ent;

int main(int argc, char** argv)
{
    unsigned const seed = argc > 1 ? unsigned(std::atoi(argv[1])) : 1u;
    long const cases = argc > 2 ? std::atol(argv[2]) : 20000;
    std::mt19937_64 rng(seed);
    long bad = 0, fseCases = 0, hufCases = 0;
    for (long c = 0; c < cases; c++) {
        unsigned count[256] = {};
        unsigned const maxSym = 1 + unsigned(rng() % 255);
        uint64_t const total = 2 + rng() % (rng() % 4 == 0 ? 200 : 100000);
        int const shape = int(rng() % 6);
        double const zs = 1.0 + double(rng() % 1000) / 500.0;
        for (uint64_t i = 0; i < total; i++) {
            unsigned s = 0;
            switch (shape) {
                case 0: s = unsigned(rng() % (maxSym + 1)); break;                      // uniform
                case 1: {                                                                // Zipf-like
                    double const u = double(rng() % 1000000 + 1) / 1000001.0;
                    s = unsigned(double(maxSym + 1) * std::pow(u, zs * 2.0));
                    break;
                }
                case 2: { unsigned g = 0; while (g < maxSym && rng() % 3 != 0) g++; s = g; break; } // geometric
                case 3: s = rng() % 20 ? 0u : unsigned(rng() % (maxSym + 1)); break;   // one dominant symbol
                case 4: s = unsigned((rng() % 8) * (maxSym / 7 + 1)) % (maxSym + 1); break; // sparse
                default: s = rng() % 2 ? unsigned(rng() % 4) : unsigned(rng() % (maxSym + 1)); break; // many rare
            }
            if (s > maxSym) s = maxSym;
            count[s]++;
        }
        if (rng() % 4 == 0) {
            // groups of equal counts around the bucket cutoff (9 to 40 symbols
            // of one count in 160..170, or of a random count): the order the
            // reference's sort leaves equal counts in decides the codes
            uint32_t const v = rng() % 2 ? 160 + uint32_t(rng() % 11) : 1 + uint32_t(rng() % 5000);
            unsigned const k = 9 + unsigned(rng() % 32);
            for (unsigned q = 0; q < k; q++) count[rng() % (maxSym + 1)] = v;
        }
        count[maxSym] += 1; // the largest symbol is present
        uint64_t tot = 0;
        unsigned distinct = 0;
        for (unsigned s = 0; s <= maxSym; s++) {
            tot += count[s];
            distinct += count[s] != 0;
        }
        if (distinct < 2) continue; // a single symbol is not entropy-coded
        // FSE: table log (the encoder's maximum 11, and 12), counts, header
        for (unsigned maxTL : { 11u, 12u }) {
            unsigned const tlRef = ZS_FSE_optimalTableLog_internal(maxTL, size_t(tot), maxSym, 2);
            unsigned const tl = fseTableLogOf(maxTL, tot, maxSym, 2);
            if (tl != tlRef) { bad++; std::printf("BAD fse tl %u ref %u (n=%llu max=%u)\n", tl, tlRef, (unsigned long long)tot, maxSym); continue; }
            short normRef[256] = {};
            size_t const r = ZS_FSE_normalizeCount(normRef, tl, count, size_t(tot), maxSym, 1);
            int16_t norm[256] = {};
            bool const ok = fseNormalizeCounts(norm, tl, count, tot, maxSym);
            if (ZS_FSE_isError(r) || !ok) {
                if (ZS_FSE_isError(r) != !ok) { bad++; std::printf("BAD fse normalize outcome\n"); }
                continue;
            }
            fseCases++;
            for (unsigned s = 0; s <= maxSym; s++)
                if (norm[s] != normRef[s]) { bad++; std::printf("BAD fse norm[%u] %d ref %d\n", s, norm[s], normRef[s]); break; }
            uint8_t hdr[600] = {}, hdrRef[600] = {};
            size_t const hs = fseWriteNCountTo(hdr, norm, maxSym, tl);
            size_t const hr = ZS_FSE_writeNCount(hdrRef, sizeof hdrRef, normRef, maxSym, tl);
            if (ZS_FSE_isError(hr) || hs != hr || std::memcmp(hdr, hdrRef, hs) != 0) { bad++; std::printf("BAD fse header %zu ref %zu\n", hs, hr); }
        }
        // Huffman: table log, code lengths and codes
        {
            unsigned const tlRef = ZS_FSE_optimalTableLog_internal(11, size_t(tot), maxSym, 1);
            unsigned const tl = fseTableLogOf(11, tot, maxSym, 1);
            if (tl != tlRef) { bad++; std::printf("BAD huf tl %u ref %u\n", tl, tlRef); continue; }
            std::vector<size_t> ct(maxSym + 2, 0);
            size_t const mr = ZS_HUF_buildCTable(ct.data(), count, maxSym, tl);
            static HufNode nodes[kHufNodes];
            uint16_t value[256];
            uint8_t nbBits[256];
            unsigned const mb = hufBuildCodes(nodes, value, nbBits, count, maxSym, tl);
            if (ZS_HUF_isError(mr)) { bad++; std::printf("BAD huf reference error\n"); continue; }
            hufCases++;
            if (mb != unsigned(mr)) { bad++; std::printf("BAD huf maxNbBits %u ref %zu\n", mb, mr); }
            for (unsigned s = 0; s <= maxSym; s++) {
                size_t const e = ct[1 + s];
                unsigned const nb = unsigned(e & 0xFF);
                unsigned const v = nb ? unsigned(e >> (8 * sizeof(size_t) - nb)) : 0u;
                if (nb != nbBits[s] || (nb && v != value[s])) {
                    bad++;
                    std::printf("BAD huf sym %u: %u/%u ref %u/%u\n", s, nbBits[s], value[s], nb, v);
                    break;
                }
            }
        }
    }
    // 16-bit symbols (huffman_struct_v2): code lengths and codes against
    // ZS_largeHuffmanBuildCTable with the binding's table log (0: 20), on
    // large alphabets and groups of equal counts
    long huf16Cases = 0;
    for (long c = 0; c < cases / 8; c++) {
        unsigned const maxSym = 1 + unsigned(rng() % (rng() % 4 == 0 ? 65535 : 3000));
        std::vector<uint32_t> count(maxSym + 1, 0);
        uint64_t const total = 2 + rng() % 200000;
        int const shape = int(rng() % 4);
        for (uint64_t i = 0; i < total; i++) {
            unsigned s = 0;
            switch (shape) {
                case 0: s = unsigned(rng() % (maxSym + 1)); break;
                case 1: {
                    double const u = double(rng() % 1000000 + 1) / 1000001.0;
                    s = unsigned(double(maxSym + 1) * u * u * u);
                    break;
                }
                case 2: { unsigned g = 0; while (g < maxSym && rng() % 4 != 0) g++; s = g; break; }
                default: s = rng() % 2 ? unsigned(rng() % 64) : unsigned(rng() % (maxSym + 1)); break;
            }
            count[s > maxSym ? maxSym : s]++;
        }
        if (rng() % 3 == 0) {
            uint32_t const v = 1 + uint32_t(rng() % 400);
            unsigned const k = 2 + unsigned(rng() % 60);
            for (unsigned q = 0; q < k; q++) count[rng() % (maxSym + 1)] = v;
        }
        count[maxSym] += 1;
        unsigned distinct = 0;
        for (uint32_t x : count) distinct += x != 0;
        if (distinct < 2) continue;
        std::vector<RefHuf16CElt> ct(maxSym + 1, RefHuf16CElt{ 0, 0 });
        std::vector<unsigned> cnt(count.begin(), count.end());
        RefReport const rr = ZS_largeHuffmanBuildCTable(ct.data(), cnt.data(), uint16_t(maxSym), 0);
        std::vector<uint16_t> code(maxSym + 1, 0);
        std::vector<uint8_t> nbb(maxSym + 1, 0);
        int const tl = ozl::ent::huf16Build(code.data(), nbb.data(), count.data(), maxSym);
        if (rr.code != 0 || tl < 0) {
            if ((rr.code != 0) != (tl < 0)) { bad++; std::printf("BAD huf16 outcome %d %d\n", rr.code, tl); }
            continue;
        }
        huf16Cases++;
        if (size_t(tl) != rr.value) { bad++; std::printf("BAD huf16 tableLog %d ref %zu\n", tl, rr.value); continue; }
        for (unsigned s = 0; s <= maxSym; s++)
            if (ct[s].nbBits != nbb[s] || (nbb[s] && ct[s].symbol != code[s])) {
                bad++;
                std::printf("BAD huf16 sym %u: %u/%u ref %u/%u (max %u)\n", s, nbb[s], code[s], ct[s].nbBits,
                            ct[s].symbol, maxSym);
                break;
            }
    }
    // the codec decision's estimates (entropyCompressChunk compares them):
    // entropy bit for bit, fast Huffman, flat-packed and bit-packed sizes,
    // cardinality and largest symbol, on random byte arrays
    long statCases = 0;
    alignas(64) static unsigned char statsBlock[16384];
    for (long c = 0; c < cases / 8; c++) {
        size_t const n = 1 + size_t(rng() % (rng() % 4 == 0 ? 64 : 200000));
        std::vector<uint8_t> src(n);
        unsigned const alpha = 1 + unsigned(rng() % 256);
        int const shape = int(rng() % 4);
        for (size_t i = 0; i < n; i++) {
            unsigned v = 0;
            switch (shape) {
                case 0: v = unsigned(rng() % alpha); break;
                case 1: { double const u = double(rng() % 1000000) / 1000000.0; v = unsigned(double(alpha) * u * u); break; }
                case 2: v = rng() % 50 ? 7u : unsigned(rng() % alpha); break;
                default: v = unsigned((i / (1 + rng() % 64)) % alpha); break;
            }
            src[i] = uint8_t(v);
        }
        ozl::ent::Histo h{};
        for (uint8_t v : src) h.count[v]++;
        h.n = n;
        h.finish();
        std::memset(statsBlock, 0, sizeof statsBlock);
        DataStatsU8_init(statsBlock, src.data(), n);
        double const eRef = DataStatsU8_getEntropy(statsBlock);
        double const eRef2 = ZL_calculateEntropyU8(h.count, n);
        double const e = ozl::ent::entropyEstimate(h.count, n);
        statCases++;
        if (std::memcmp(&e, &eRef, sizeof e) != 0 || std::memcmp(&e, &eRef2, sizeof e) != 0) {
            bad++;
            std::printf("BAD entropy %.17g ref %.17g / %.17g (n=%zu)\n", e, eRef, eRef2, n);
            continue;
        }
        uint64_t const hf = ozl::ent::hufSizeFast(e, n), hfRef = DataStatsU8_estimateHuffmanSizeFast(statsBlock, false);
        uint64_t const fp = ozl::ent::flatpackedSize(h), fpRef = DataStatsU8_getFlatpackedSize(statsBlock);
        uint64_t const bp = ozl::ent::bitpackedSize(h), bpRef = DataStatsU8_getBitpackedSize(statsBlock);
        if (hf != hfRef || fp != fpRef || bp != bpRef || h.card != DataStatsU8_getCardinality(statsBlock)
            || h.maxSym != DataStatsU8_getMaxElt(statsBlock)) {
            bad++;
            std::printf("BAD stats n=%zu huf %llu/%llu flat %llu/%llu bit %llu/%llu\n", n, (unsigned long long)hf,
                        (unsigned long long)hfRef, (unsigned long long)fp, (unsigned long long)fpRef,
                        (unsigned long long)bp, (unsigned long long)bpRef);
        }
    }
    std::printf("fse=%ld huf=%ld huf16=%ld stats=%ld bad=%ld\n", fseCases, hufCases, huf16Cases, statCases, bad);
    return bad ? 1 : 0;
}
