// Huffman code lengths and canonical codes of one chunk, shared by the host
// path and the device table builder (kHufTables). They restate
// src/openzl/fse/compress/huf_compress.c exactly (the lengths decide the
// frame's bytes): HUF_sort (:352-420, bucket sort with a quicksort of the
// large-count buckets), HUF_buildTree (:580-640), HUF_setMaxHeight
// (:430-560) and HUF_buildCTableFromTree (:700-760). The quicksort runs on an
// explicit stack: partitions of disjoint ranges do not interact, so the
// result is that of the recursive order. Integer arithmetic only.
#pragma once
#include <cstdint>

#include "fse_norm.h"

namespace ozl {
namespace ent {

struct HufNode {
    uint32_t count;
    uint16_t parent;
    uint8_t byte;
    uint8_t nbBits;
};

// 514 nodes: a sentinel, 256 leaves sorted by decreasing count, the inner nodes
constexpr int kHufNodes = 2 * 256 + 2;

// Rank buckets of HUF_sort (huf_compress.c:484-509): counts below the
// distinct-count cutoff have a bucket each, larger counts one per power of
// two from bucket 158 + highbit. The cutoff is 158 + highbit32(158) = 165
// (the reference's comment says 166; its macro arithmetic gives 165), and
// HUF_sort quicksorts the rank buckets from 165 on: rank r holds index
// r - 1, so the bucket of count 164 is quicksorted too, which reorders
// equal counts.
constexpr uint32_t kHufDistinctCutoff = 165;
OZL_HD inline uint32_t hufBucketOf(uint32_t c)
{
    return c < kHufDistinctCutoff ? c : uint32_t(highbit32v(c)) + 158;
}

OZL_HD inline void hufInsertionSort(HufNode* a, int low, int high)
{
    a += low;
    int const size = high - low + 1;
    for (int i = 1; i < size; i++) {
        HufNode const key = a[i];
        int j = i - 1;
        while (j >= 0 && a[j].count < key.count) {
            a[j + 1] = a[j];
            j--;
        }
        a[j + 1] = key;
    }
}

OZL_HD inline int hufPartitionDesc(HufNode* a, int low, int high)
{
    uint32_t const pivot = a[high].count;
    int i = low - 1;
    for (int j = low; j < high; j++)
        if (a[j].count > pivot) {
            i++;
            HufNode t = a[i];
            a[i] = a[j];
            a[j] = t;
        }
    HufNode t = a[i + 1];
    a[i + 1] = a[high];
    a[high] = t;
    return i + 1;
}

// Descending quicksort as the reference recurses: a call on a range under 8
// elements insertion-sorts it; otherwise it partitions, calls itself on the
// smaller side, and keeps partitioning the larger side (without the size
// check) until the range is empty. The stack holds calls and loop
// continuations; the smaller side runs first, so the stack stays within
// 2 log2(256) + 2 entries.
OZL_HD inline void hufQuickSortDesc(HufNode* a, int low0, int high0)
{
    int stk[3 * 40];
    int sp = 0;
    auto push = [&](int kind, int lo, int hi) {
        stk[sp++] = kind;
        stk[sp++] = lo;
        stk[sp++] = hi;
    };
    push(0, low0, high0);
    while (sp) {
        int high = stk[--sp];
        int low = stk[--sp];
        int const kind = stk[--sp];
        if (kind == 0 && high - low < 8) {
            hufInsertionSort(a, low, high);
            continue;
        }
        if (low < high) {
            int const idx = hufPartitionDesc(a, low, high);
            if (idx - low < high - idx) {
                push(1, idx + 1, high); // the loop continues on the larger side
                push(0, low, idx - 1);  // after the call on the smaller side
            } else {
                push(1, low, idx - 1);
                push(0, idx + 1, high);
            }
        }
    }
}

OZL_HD inline void hufSortByCount(HufNode* node, const uint32_t* count, unsigned maxSym)
{
    uint16_t base[192], curr[192];
    for (int n = 0; n < 192; n++) base[n] = curr[n] = 0;
    for (unsigned n = 0; n <= maxSym; n++) base[hufBucketOf(count[n])]++;
    for (int n = 191; n > 0; n--) {
        base[n - 1] = uint16_t(base[n - 1] + base[n]);
        curr[n - 1] = base[n - 1];
    }
    for (unsigned n = 0; n <= maxSym; n++) {
        uint32_t const pos = curr[hufBucketOf(count[n]) + 1]++;
        node[pos].count = count[n];
        node[pos].byte = uint8_t(n);
    }
    for (int n = int(kHufDistinctCutoff); n < 191; n++) {
        int const size = curr[n] - base[n];
        if (size > 1) hufQuickSortDesc(node + base[n], 0, size - 1);
    }
}

OZL_HD inline uint32_t hufLimitHeight(HufNode* node, uint32_t last, uint32_t target)
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
    for (int k = 0; k < 14; k++) rankLast[k] = none;
    uint32_t cur = target;
    for (int pos = n; pos >= 0; pos--) {
        if (node[pos].nbBits >= cur) continue;
        cur = node[pos].nbBits;
        rankLast[target - cur] = uint32_t(pos);
    }
    while (cost > 0) {
        uint32_t k = uint32_t(highbit32v(uint32_t(cost))) + 1;
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

// Code lengths and codes of symbols 0..maxSym (at least two of them with a
// nonzero count) in `all` (kHufNodes nodes of scratch): nbBits[] and value[]
// of 256 entries (0 for absent symbols). Returns the table log.
OZL_HD inline unsigned hufBuildCodes(HufNode* all, uint16_t* value, uint8_t* nbBitsOut, const uint32_t* count,
                                     unsigned maxSym, unsigned maxNbBits)
{
    for (int k = 0; k < kHufNodes; k++) all[k] = HufNode{ 0, 0, 0, 0 };
    HufNode* node = all + 1;
    hufSortByCount(node, count, maxSym);
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
    unsigned const maxBits = hufLimitHeight(node, uint32_t(nonNull), maxNbBits);
    uint16_t perRank[13], valRank[13];
    for (int k = 0; k < 13; k++) perRank[k] = valRank[k] = 0;
    for (int n = 0; n <= nonNull; n++) perRank[node[n].nbBits]++;
    uint16_t mn = 0;
    for (int n = int(maxBits); n > 0; n--) {
        valRank[n] = mn;
        mn = uint16_t((mn + perRank[n]) >> 1);
    }
    for (int k = 0; k < 256; k++) {
        value[k] = 0;
        nbBitsOut[k] = 0;
    }
    for (unsigned n = 0; n <= maxSym; n++) nbBitsOut[node[n].byte] = node[n].nbBits;
    for (unsigned n = 0; n <= maxSym; n++) value[n] = valRank[nbBitsOut[n]]++;
    return maxBits;
}

} // namespace ent
} // namespace ozl
