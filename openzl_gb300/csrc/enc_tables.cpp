// Host-side entropy decisions and coding tables (see enc_tables.h).
#include "enc_tables.h"
#include "fse_norm.h"
#include "huf_tree.h"

#include <cmath>
#include <cstring>
#include <vector>
#include <algorithm>

namespace ozl {
namespace ent {

namespace {

int highbit32(uint32_t v) { return 31 - __builtin_clz(v); }

// Integer log2 table of the entropy estimate: entry i holds
// 0x80000 ^ int(log2(256 + i) * 2^16), the generating formula stated with the
// reference table (src/openzl/shared/data_stats.c:15-18).
struct Log2Table {
    uint16_t v[256];
    Log2Table()
    {
        for (int i = 0; i < 256; i++) v[i] = uint16_t(0x80000 ^ int(std::log2(double(256 + i)) * 65536.0));
    }
};
const Log2Table kLog2;

// ZL_calculateEntropy (src/openzl/shared/data_stats.c:46-79) over values
// 0..maxValue.
double entropyBits(const uint32_t* count, uint64_t total, unsigned maxValue = 255)
{
    if (total == 0) return 0;
    int64_t acc = 0;
    int64_t const normalize = (int64_t(1) << 62) / int64_t(total);
    for (unsigned i = 0; i <= maxValue; i++) {
        int64_t const c = count[i];
        int64_t idx = c * normalize;
        int const clz = __builtin_clzll(uint64_t(idx) | (1u << 9));
        idx >>= (62 - 8) - clz + 1;
        idx &= 255;
        acc += -c * (int64_t(kLog2.v[idx]) - int64_t(clz) * 65536);
    }
    // Two separately rounded IEEE operations, as the reference computes them.
    volatile double num = double(acc);
    volatile double den = double(total * 65536);
    volatile double q = num / den;
    return q - 1;
}

} // namespace

int nextPow2Bits(uint64_t v)
{
    int n = 0;
    while (n < 64 && (uint64_t(1) << n) < v) n++;
    return n;
}

void Histo::finish()
{
    maxSym = 0;
    card = 0;
    for (int s = 0; s < 256; s++)
        if (count[s]) {
            card++;
            maxSym = unsigned(s);
        }
}

double entropyEstimate(const uint32_t* count, uint64_t total) { return entropyBits(count, total); }

// DataStatsU8_estimateHuffmanSizeFast (data_stats.c:287-301)
uint64_t hufSizeFast(double e, uint64_t n)
{
    if (e > 7) return n;
    double const e1 = e < 1 ? 1 : e;
    volatile double prod = e1 * double(n);
    volatile double q = prod / 8;
    return uint64_t(q);
}

// DataStatsU8_getFlatpackedSize and DataStatsU8_getBitpackedSize
// (data_stats.c:301-333)
uint64_t flatpackedSize(const Histo& h) { return (h.n * uint64_t(nextPow2Bits(h.card)) + 7) / 8 + h.card; }
uint64_t bitpackedSize(const Histo& h) { return (h.n * uint64_t(nextPow2Bits(h.maxSym + 1)) + 7) / 8; }

// entropyCompressChunk's codec choice for serial chunks
// (encode_entropy_binding.c:664-736).
ChunkCodec chooseCodec(const Histo& h, int mode)
{
    uint64_t const n = h.n;
    if (n <= 1) return CC_STORE;
    if (h.card == 1) return CC_CONSTANT;
    uint64_t entropySize;
    double const e = entropyBits(h.count, n);
    if (mode == EM_HUF) {
        entropySize = hufSizeFast(e, n);
    } else {
        volatile double prod = e * double(n);
        volatile double sum = prod + 7;
        entropySize = uint64_t(sum) / 8;
    }
    uint64_t const header = h.card / 4 > 10 ? h.card / 4 : 10;
    uint64_t baseline = entropySize + header;
    if (n < baseline) baseline = n;
    uint64_t const flat = flatpackedSize(h);
    uint64_t const bp = bitpackedSize(h);
    if (flat < bp) {
        if (flat < baseline) return CC_FLATPACK;
    } else if (bp < baseline) {
        return CC_BITPACK;
    }
    if (n <= baseline) return CC_STORE;
    // resolveMode (encode_entropy_binding.c:527-548): the FSE size is the
    // entropy estimate above
    if (mode == EM_ANY) return entropySize + n / 32 < hufSizeFast(e, n) ? CC_FSE : CC_HUF;
    return mode == EM_HUF ? CC_HUF : CC_FSE;
}

// FSE table log, normalization and header: the shared restatement in
// fse_norm.h (the device table builder uses the same functions)
unsigned fseTableLog(unsigned maxTL, uint64_t srcSize, unsigned maxSym, unsigned minus)
{
    return fseTableLogOf(maxTL, srcSize, maxSym, minus);
}

bool fseNormalize(int16_t* norm, unsigned tl, const uint32_t* count, uint64_t total, unsigned maxSym)
{
    return fseNormalizeCounts(norm, tl, count, total, maxSym);
}

size_t fseWriteNCount(uint8_t* out, const int16_t* norm, unsigned maxSym, unsigned tl)
{
    return fseWriteNCountTo(out, norm, maxSym, tl);
}

// FSE_buildCTable_wksp (fse_compress.c:69-207)
void fseBuildCTable(FseCTable& ct, const int16_t* norm, unsigned maxSym, unsigned tl)
{
    uint32_t const size = 1u << tl, mask = size - 1, step = (size >> 1) + (size >> 3) + 3;
    uint16_t cumul[258];
    uint8_t symbolAt[4096];
    uint32_t high = size - 1;
    ct.tableLog = uint16_t(tl);
    ct.maxSym = uint16_t(maxSym);
    cumul[0] = 0;
    for (unsigned u = 1; u <= maxSym + 1; u++) {
        if (norm[u - 1] == -1) {
            cumul[u] = uint16_t(cumul[u - 1] + 1);
            symbolAt[high--] = uint8_t(u - 1);
        } else {
            cumul[u] = uint16_t(cumul[u - 1] + uint16_t(norm[u - 1]));
        }
    }
    uint32_t pos = 0;
    for (unsigned s = 0; s <= maxSym; s++)
        for (int i = 0; i < norm[s]; i++) {
            symbolAt[pos] = uint8_t(s);
            do { pos = (pos + step) & mask; } while (pos > high);
        }
    for (uint32_t u = 0; u < size; u++) ct.state[cumul[symbolAt[u]]++] = uint16_t(size + u);
    unsigned total = 0;
    for (unsigned s = 0; s < 256; s++) {
        int const c = s <= maxSym ? norm[s] : 0;
        fseSymbolDeltas(c, tl, total, ct.deltaNbBits[s], ct.deltaFindState[s]);
        total += c == -1 ? 1u : unsigned(c);
    }
}

// ---------------------------------------------------------------------------
// Huffman code lengths and codes: the shared restatement in huf_tree.h (the
// device table builder uses the same functions)
unsigned hufBuild(HufCTable& ct, const uint32_t* count, unsigned maxSym, unsigned maxNbBits)
{
    HufNode all[kHufNodes];
    unsigned const tl = hufBuildCodes(all, ct.value, ct.nbBits, count, maxSym, maxNbBits);
    ct.tableLog = tl;
    return tl;
}

// ---------------------------------------------------------------------------
// 16-bit chunks

ChunkCodec chooseCodec16(const uint32_t* count, unsigned maxSym, uint64_t n, unsigned card)
{
    if (count[maxSym] == n) return CC_CONSTANT;
    double entropy = entropyBits(count, n, maxSym);
    if (1 > entropy) entropy = 1;
    volatile double prod = entropy * double(n);
    volatile double sum = prod + 7;
    uint64_t const entropySize = uint64_t(sum) / 8;
    uint64_t const header = maxSym / 4 > 100 ? maxSym / 4 : 100;
    uint64_t const huffSize = entropySize + header, storeSize = 2 * n;
    uint64_t const nbBits = uint64_t(nextPow2Bits(uint64_t(maxSym) + 1));
    uint64_t const bitpackSize = (n * nbBits + 7) / 8 + 2;
    if (bitpackSize <= huffSize && bitpackSize < storeSize) return CC_BITPACK;
    if (entropy > 15 || huffSize >= storeSize) return CC_STORE;
    if (card < 256) return CC_TOK16;
    return CC_HUF16;
}

namespace {

struct LNode {
    uint32_t count, parent;
    uint16_t symbol, nbBits;
};

// ZS_largeHuffmanSetMaxHeight (encode_huffman_kernel.c:34-151)
int huf16MaxHeight(LNode* node, int last, int maxNbBits)
{
    int const largest = node[last].nbBits;
    if (largest <= maxNbBits) return largest;
    int totalCost = 0;
    int const baseCost = 1 << (largest - maxNbBits);
    int n;
    for (n = last; node[n].nbBits > maxNbBits; --n) {
        totalCost += baseCost - (1 << (largest - node[n].nbBits));
        node[n].nbBits = uint16_t(maxNbBits);
    }
    while (node[n].nbBits == maxNbBits) --n;
    totalCost >>= (largest - maxNbBits);
    uint32_t const noSym = 0xF0F0F0F0u;
    uint32_t rankLast[22];
    for (uint32_t& r : rankLast) r = noSym;
    {
        int cur = maxNbBits;
        for (int pos = n; pos >= 0; pos--) {
            if (node[pos].nbBits >= cur) continue;
            cur = node[pos].nbBits;
            rankLast[maxNbBits - cur] = uint32_t(pos);
        }
    }
    while (totalCost > 0) {
        int nb = highbit32(uint32_t(totalCost)) + 1;
        while (nb > 1 && rankLast[nb] == noSym) --nb;
        for (; nb > 1; nb--) {
            uint32_t const hi = rankLast[nb], lo = rankLast[nb - 1];
            if (hi == noSym || lo == noSym) break;
            if (node[hi].count <= 2 * node[lo].count) break;
        }
        while (nb <= 20 && rankLast[nb] == noSym) nb++;
        if (nb > 21 || rankLast[nb] == noSym) return -1;
        totalCost -= 1 << (nb - 1);
        if (rankLast[nb - 1] == noSym) rankLast[nb - 1] = rankLast[nb];
        node[rankLast[nb]].nbBits++;
        if (rankLast[nb] == 0) {
            rankLast[nb] = noSym;
        } else {
            rankLast[nb]--;
            if (node[rankLast[nb]].nbBits != maxNbBits - nb) rankLast[nb] = noSym;
        }
    }
    while (totalCost < 0) {
        if (rankLast[1] == noSym) {
            while (node[n].nbBits == maxNbBits) n--;
            node[n + 1].nbBits--;
            rankLast[1] = uint32_t(n + 1);
            totalCost++;
            continue;
        }
        node[rankLast[1] + 1].nbBits--;
        rankLast[1]++;
        totalCost++;
    }
    return maxNbBits;
}

} // namespace

int huf16Build(uint16_t* code, uint8_t* nbBits, const uint32_t* count, unsigned maxSym)
{
    int maxNbBits = 20;
    int const bound = nextPow2Bits(uint64_t(maxSym) + 1);
    if (bound + 3 < maxNbBits) maxNbBits = bound + 3;
    std::vector<LNode> all(2 * size_t(maxSym) + 3, LNode{ 0, 0, 0, 0 });
    LNode* const node = all.data() + 1;
    for (unsigned s = 0; s <= maxSym; s++) node[s] = LNode{ count[s], 0, uint16_t(s), 0 };
    // ZS_largeHuffmanSort (encode_huffman_kernel.c:153-229): decreasing
    // counts; the reference's partition by highest set bit is stable, so
    // equal counts keep symbol order
    std::stable_sort(node, node + maxSym + 1, [](const LNode& a, const LNode& b) { return a.count > b.count; });
    // ZS_largeHuffmanBuildTree (encode_huffman_kernel.c:231-290); node[-1]
    // is the sentinel
    int nonNull = int(maxSym);
    while (node[nonNull].count == 0) nonNull--;
    int const startNode = int(maxSym) + 1;
    int nodeNb = startNode, lowS = nonNull, lowN = nodeNb;
    int const nodeRoot = nodeNb + lowS - 1;
    node[nodeNb].count = node[lowS].count + node[lowS - 1].count;
    node[lowS].parent = node[lowS - 1].parent = uint32_t(nodeNb);
    nodeNb++;
    lowS -= 2;
    for (int k = nodeNb; k <= nodeRoot; k++) node[k].count = 1u << 30;
    node[-1].count = 1u << 31;
    for (; nodeNb <= nodeRoot; nodeNb++) {
        int const n1 = node[lowS].count < node[lowN].count ? lowS-- : lowN++;
        int const n2 = node[lowS].count < node[lowN].count ? lowS-- : lowN++;
        node[nodeNb].count = node[n1].count + node[n2].count;
        node[n1].parent = node[n2].parent = uint32_t(nodeNb);
    }
    node[nodeRoot].nbBits = 0;
    for (int k = nodeRoot - 1; k >= startNode; k--) node[k].nbBits = uint16_t(node[node[k].parent].nbBits + 1);
    for (int k = 0; k <= nonNull; k++) node[k].nbBits = uint16_t(node[node[k].parent].nbBits + 1);
    maxNbBits = huf16MaxHeight(node, nonNull, maxNbBits);
    if (maxNbBits < 0 || maxNbBits > 20) return -1;
    // canonical codes (ZS_largeHuffmanBuildCTableFromTree, 16-bit arithmetic)
    uint16_t nbPerRank[21] = { 0 }, valPerRank[21] = { 0 };
    for (int k = 0; k <= nonNull; k++) nbPerRank[node[k].nbBits]++;
    uint16_t mn = 0;
    for (int k = maxNbBits; k > 0; k--) {
        valPerRank[k] = mn;
        mn = uint16_t(mn + nbPerRank[k]);
        mn >>= 1;
    }
    for (unsigned k = 0; k <= maxSym; k++) nbBits[node[k].symbol] = uint8_t(node[k].nbBits);
    for (unsigned s = 0; s <= maxSym; s++) code[s] = valPerRank[nbBits[s]]++;
    return maxNbBits;
}

} // namespace ent
} // namespace ozl
