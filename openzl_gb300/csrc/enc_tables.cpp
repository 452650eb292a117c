// Host-side entropy decisions and coding tables (see enc_tables.h).
#include "enc_tables.h"

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

// entropyCompressChunk's codec choice for serial chunks
// (encode_entropy_binding.c:664-736).
// DataStatsU8_estimateHuffmanSizeFast (data_stats.c:287-301)
static uint64_t hufSizeFast(double e, uint64_t n)
{
    if (e > 7) return n;
    double const e1 = e < 1 ? 1 : e;
    volatile double prod = e1 * double(n);
    volatile double q = prod / 8;
    return uint64_t(q);
}

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
    uint64_t const flat = (n * uint64_t(nextPow2Bits(h.card)) + 7) / 8 + h.card;
    uint64_t const bp = (n * uint64_t(nextPow2Bits(h.maxSym + 1)) + 7) / 8;
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

// FSE_optimalTableLog_internal (fse_compress.c:379-396)
unsigned fseTableLog(unsigned maxTL, uint64_t srcSize, unsigned maxSym, unsigned minus)
{
    unsigned const maxBitsSrc = unsigned(highbit32(uint32_t(srcSize - 1))) - minus;
    unsigned const a = unsigned(highbit32(uint32_t(srcSize))) + 1;
    unsigned const b = unsigned(highbit32(maxSym)) + 2;
    unsigned const minBits = a < b ? a : b;
    unsigned tl = maxTL ? maxTL : 11;
    if (maxBitsSrc < tl) tl = maxBitsSrc;
    if (minBits > tl) tl = minBits;
    if (tl < 5) tl = 5;
    if (tl > 12) tl = 12;
    return tl;
}

namespace {
// FSE_normalizeM2 (fse_compress.c:400-470)
bool normalizeM2(int16_t* norm, unsigned tl, const uint32_t* count, uint64_t total, unsigned maxSym)
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
} // namespace

// FSE_normalizeCount with low-probability counts (fse_compress.c:472-520)
bool fseNormalize(int16_t* norm, unsigned tl, const uint32_t* count, uint64_t total, unsigned maxSym)
{
    static const uint32_t restToBeat[] = { 0, 473195, 504333, 520860, 550000, 700000, 750000, 830000 };
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
    if (-still >= (norm[largest] >> 1)) return normalizeM2(norm, tl, count, total, maxSym);
    norm[largest] = int16_t(norm[largest] + int16_t(still));
    return true;
}

// FSE_writeNCount_generic (fse_compress.c:226-338)
size_t fseWriteNCount(uint8_t* out, const int16_t* norm, unsigned maxSym, unsigned tl)
{
    size_t op = 0;
    uint32_t bits = 0;
    int nb = 0;
    int remaining = (1 << tl) + 1, threshold = 1 << tl, width = int(tl) + 1;
    unsigned sym = 0;
    unsigned const alphabet = maxSym + 1;
    bool prev0 = false;
    auto flush16 = [&]() {
        out[op] = uint8_t(bits);
        out[op + 1] = uint8_t(bits >> 8);
        op += 2;
        bits >>= 16;
    };
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
                flush16();
            }
            while (sym >= start + 3) {
                start += 3;
                bits += 3u << nb;
                nb += 2;
            }
            bits += (sym - start) << nb;
            nb += 2;
            if (nb > 16) {
                flush16();
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
            flush16();
            nb -= 16;
        }
    }
    out[op] = uint8_t(bits);
    out[op + 1] = uint8_t(bits >> 8);
    op += size_t((nb + 7) / 8);
    return op;
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
        if (c == 0) {
            ct.deltaNbBits[s] = ((tl + 1) << 16) - (1u << tl);
            ct.deltaFindState[s] = 0;
        } else if (c == -1 || c == 1) {
            ct.deltaNbBits[s] = (tl << 16) - (1u << tl);
            ct.deltaFindState[s] = int(total) - 1;
            total++;
        } else {
            uint32_t const maxBitsOut = tl - unsigned(highbit32(uint32_t(c) - 1));
            uint32_t const minStatePlus = uint32_t(c) << maxBitsOut;
            ct.deltaNbBits[s] = (maxBitsOut << 16) - minStatePlus;
            ct.deltaFindState[s] = int(total) - c;
            total += unsigned(c);
        }
    }
}

// ---------------------------------------------------------------------------
// Huffman code lengths: HUF_sort, HUF_buildTree, HUF_setMaxHeight and
// HUF_buildCTableFromTree (huf_compress.c:352-760).
namespace {
struct Node {
    uint32_t count;
    uint16_t parent;
    uint8_t byte;
    uint8_t nbBits;
};

uint32_t bucketOf(uint32_t c) { return c < 166 ? c : uint32_t(highbit32(c)) + 158; }

void insertionSort(Node* a, int low, int high)
{
    a += low;
    int const size = high - low + 1;
    for (int i = 1; i < size; i++) {
        Node const key = a[i];
        int j = i - 1;
        while (j >= 0 && a[j].count < key.count) {
            a[j + 1] = a[j];
            j--;
        }
        a[j + 1] = key;
    }
}

int partitionDesc(Node* a, int low, int high)
{
    uint32_t const pivot = a[high].count;
    int i = low - 1;
    for (int j = low; j < high; j++)
        if (a[j].count > pivot) {
            i++;
            Node t = a[i];
            a[i] = a[j];
            a[j] = t;
        }
    Node t = a[i + 1];
    a[i + 1] = a[high];
    a[high] = t;
    return i + 1;
}

void quickSortDesc(Node* a, int low, int high)
{
    if (high - low < 8) {
        insertionSort(a, low, high);
        return;
    }
    while (low < high) {
        int const idx = partitionDesc(a, low, high);
        if (idx - low < high - idx) {
            quickSortDesc(a, low, idx - 1);
            low = idx + 1;
        } else {
            quickSortDesc(a, idx + 1, high);
            high = idx - 1;
        }
    }
}

void sortByCount(Node* node, const uint32_t* count, unsigned maxSym)
{
    uint16_t base[192] = { 0 }, curr[192] = { 0 };
    for (unsigned n = 0; n <= maxSym; n++) base[bucketOf(count[n])]++;
    for (int n = 191; n > 0; n--) {
        base[n - 1] = uint16_t(base[n - 1] + base[n]);
        curr[n - 1] = base[n - 1];
    }
    for (unsigned n = 0; n <= maxSym; n++) {
        uint32_t const pos = curr[bucketOf(count[n]) + 1]++;
        node[pos].count = count[n];
        node[pos].byte = uint8_t(n);
    }
    for (int n = 166; n < 191; n++) {
        int const size = curr[n] - base[n];
        if (size > 1) quickSortDesc(node + base[n], 0, size - 1);
    }
}

uint32_t limitHeight(Node* node, uint32_t last, uint32_t target)
{
    uint32_t const largest = node[last].nbBits;
    if (largest <= target) return largest;
    int cost = 0;
    int const baseCost = 1 << (largest - target);
    int n = int(last);
    while (node[n].nbBits > target) {
        cost += baseCost - (1 << (largest - node[n].nbBits));
        node[n].nbBits = uint8_t(target);
        n--;
    }
    while (node[n].nbBits == target) --n;
    cost >>= (largest - target);
    uint32_t const none = 0xF0F0F0F0u;
    uint32_t rankLast[14];
    for (auto& r : rankLast) r = none;
    uint32_t cur = target;
    for (int pos = n; pos >= 0; pos--) {
        if (node[pos].nbBits >= cur) continue;
        cur = node[pos].nbBits;
        rankLast[target - cur] = uint32_t(pos);
    }
    while (cost > 0) {
        uint32_t k = uint32_t(highbit32(uint32_t(cost))) + 1;
        for (; k > 1; k--) {
            uint32_t const hi = rankLast[k], lo = rankLast[k - 1];
            if (hi == none) continue;
            if (lo == none) break;
            if (node[hi].count <= 2 * node[lo].count) break;
        }
        while (k <= 12 && rankLast[k] == none) k++;
        cost -= 1 << (k - 1);
        node[rankLast[k]].nbBits++;
        if (rankLast[k - 1] == none) rankLast[k - 1] = rankLast[k];
        if (rankLast[k] == 0) {
            rankLast[k] = none;
        } else {
            rankLast[k]--;
            if (node[rankLast[k]].nbBits != target - k) rankLast[k] = none;
        }
    }
    while (cost < 0) {
        if (rankLast[1] == none) {
            while (node[n].nbBits == target) n--;
            node[n + 1].nbBits--;
            rankLast[1] = uint32_t(n + 1);
            cost++;
            continue;
        }
        node[rankLast[1] + 1].nbBits--;
        rankLast[1]++;
        cost++;
    }
    return target;
}
} // namespace

unsigned hufBuild(HufCTable& ct, const uint32_t* count, unsigned maxSym, unsigned maxNbBits)
{
    Node all[2 * 256 + 2];
    std::memset(all, 0, sizeof(all));
    Node* node = all + 1;
    sortByCount(node, count, maxSym);
    int const start = 256;
    int nonNull = int(maxSym);
    while (node[nonNull].count == 0) nonNull--;
    int lowS = nonNull, nodeNb = start, lowN = start;
    int const root = start + lowS - 1;
    node[nodeNb].count = node[lowS].count + node[lowS - 1].count;
    node[lowS].parent = node[lowS - 1].parent = uint16_t(nodeNb);
    nodeNb++;
    lowS -= 2;
    for (int n = nodeNb; n <= root; n++) node[n].count = 1u << 30;
    all[0].count = 1u << 31;
    while (nodeNb <= root) {
        int const n1 = node[lowS].count < node[lowN].count ? lowS-- : lowN++;
        int const n2 = node[lowS].count < node[lowN].count ? lowS-- : lowN++;
        node[nodeNb].count = node[n1].count + node[n2].count;
        node[n1].parent = node[n2].parent = uint16_t(nodeNb);
        nodeNb++;
    }
    node[root].nbBits = 0;
    for (int n = root - 1; n >= start; n--) node[n].nbBits = uint8_t(node[node[n].parent].nbBits + 1);
    for (int n = 0; n <= nonNull; n++) node[n].nbBits = uint8_t(node[node[n].parent].nbBits + 1);
    unsigned const maxBits = limitHeight(node, uint32_t(nonNull), maxNbBits);
    uint16_t perRank[13] = { 0 }, valRank[13] = { 0 };
    for (int n = 0; n <= nonNull; n++) perRank[node[n].nbBits]++;
    uint16_t mn = 0;
    for (int n = int(maxBits); n > 0; n--) {
        valRank[n] = mn;
        mn = uint16_t((mn + perRank[n]) >> 1);
    }
    std::memset(&ct, 0, sizeof(ct));
    for (unsigned n = 0; n <= maxSym; n++) ct.nbBits[node[n].byte] = node[n].nbBits;
    for (unsigned n = 0; n <= maxSym; n++) ct.value[n] = valRank[ct.nbBits[n]]++;
    ct.tableLog = maxBits;
    return maxBits;
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
