/* CPU restatement of the OpenZL compressor for the numeric graph recipes
 * (test infrastructure only: the checker for the GPU encoder, and the source
 * of reference-identical frames where the reference library is absent).
 *
 * The engine mirrors the reference's runtime graph (src/openzl/compress/
 * cctx.c:700-1230, rtgraphs.c): a graph function creates nodes immediately
 * (their output streams get consecutive stream ids), registers successor
 * graphs for its edges, and the successors then run depth-first in
 * registration order; any single successor input under 10 bytes is stored
 * instead (cctx.c:1125-1140); inputs whose type a graph does not accept get
 * an implicit conversion node first (cctx.c:563-604, implicit_conversion.c).
 * The frame lists decoders in reverse node-creation order and stored streams
 * in reverse stream-id order (cctx.c:1447-1700, rtgraphs.c:444-468).
 */
#include <math.h>
#include <stdio.h>

#include "ozo_internal.h"

/* ------------------------------------------------------------------ */
/* recipe numbers (same as oracle/ref_driver.c) */
enum {
    R_STORE = 0, R_DZ_TSPLIT_FSE = 1, R_DZ_BITPACK_HUF = 2, R_D_TSPLIT_FSE = 3,
    R_D_BITPACK_HUF = 4, R_TOKENIZE = 5, R_BF16 = 6, R_FSE = 7, R_HUFFMAN = 8,
    R_DELTA_STORE = 9, R_ZIGZAG_STORE = 10, R_BITPACK_STORE = 11, R_TSPLIT_STORE = 12,
    R_CONSTANT = 13, R_FLATPACK = 14, R_BITPACK_GRAPH = 15, R_TOKENIZE_SORTED = 16,
    R_ENTROPY = 17,
};

/* graphs of the engine */
enum {
    G_STORE, G_SERIAL_STORE, G_FSE, G_HUF, G_CONSTANT, G_BITPACK, G_FLATPACK, G_FSE_NCOUNT,
    G_TSPLIT_FSE, G_TSPLIT_STORE, G_BITPACK_HUF, G_CHAIN, G_TOKENIZE, G_TOKENIZE_SORTED, G_BF16,
    G_ENTROPY,
};

typedef struct {
    int type;
    size_t w, n;
    uint8_t* data; /* owned copy of the content */
    int store;
} EStream;

typedef struct {
    unsigned trid;
    uint8_t hdr[16];
    size_t hsz;
    int in;          /* encoder input stream (single-input codecs only) */
    int outStart, nbOut, nbSO;
} ENode;

typedef struct {
    EStream* s;
    size_t ns, cs;
    ENode* nd;
    size_t nn, cn;
    int err;
} ECtx;

static int new_stream(ECtx* c, int type, size_t w, size_t n, const uint8_t* src)
{
    if (c->ns == c->cs) {
        c->cs = c->cs ? 2 * c->cs : 64;
        c->s = (EStream*)realloc(c->s, c->cs * sizeof(EStream));
    }
    EStream* s = &c->s[c->ns];
    s->type = type;
    s->w = w;
    s->n = n;
    s->data = (uint8_t*)malloc(n * w + 16);
    if (src && n) memcpy(s->data, src, n * w);
    s->store = 0;
    return (int)c->ns++;
}

static ENode* new_node(ECtx* c, unsigned trid, int in, int nbSO)
{
    if (c->nn == c->cn) {
        c->cn = c->cn ? 2 * c->cn : 64;
        c->nd = (ENode*)realloc(c->nd, c->cn * sizeof(ENode));
    }
    ENode* n = &c->nd[c->nn++];
    memset(n, 0, sizeof(*n));
    n->trid = trid;
    n->in = in;
    n->outStart = (int)c->ns;
    n->nbSO = nbSO;
    return n;
}

#define S(i) (&c->s[(i)])

/* ------------------------------------------------------------------ */
/* small helpers */
static uint64_t rd(const uint8_t* p, size_t w) { return ozo_rdN(p, w); }
static void wr(uint8_t* p, uint64_t v, size_t w)
{
    for (size_t b = 0; b < w; b++) p[b] = (uint8_t)(v >> (8 * b));
}

/* ------------------------------------------------------------------ */
/* histogram statistics (src/openzl/shared/data_stats.c) */
static uint16_t gLog2[256];
static int gLog2Init = 0;
/* LOG2_TABLE[i] = 0x80000 ^ int(log2(256 + i) * 65536): the table's stated
 * generating formula (data_stats.c:15-18). */
static void init_log2(void)
{
    if (gLog2Init) return;
    for (int i = 0; i < 256; i++) gLog2[i] = (uint16_t)(0x80000 ^ (int)(log2((double)(256 + i)) * 65536.0));
    gLog2Init = 1;
}

/* ZL_calculateEntropy (data_stats.c:46-79): integer log approximation,
 * then one double division. */
static double calc_entropy(const unsigned* count, size_t maxValue, size_t total)
{
    init_log2();
    if (total == 0) return 0;
    int64_t intEntropy = 0;
    int64_t const normalize = ((int64_t)1 << 62) / (int64_t)total;
    for (size_t i = 0; i <= maxValue; i++) {
        unsigned const cc = count[i];
        int64_t logIndex = (int64_t)(cc * normalize);
        int const clz = __builtin_clzll((uint64_t)logIndex | (1u << 9));
        int const shift = (62 - 8) - clz + 1;
        logIndex >>= shift;
        logIndex &= 255;
        intEntropy += -(int64_t)cc * ((int64_t)gLog2[logIndex] - (int64_t)clz * 65536);
    }
    volatile double num = (double)intEntropy;
    volatile double den = (double)(total * 65536);
    volatile double q = num / den;
    return q - 1;
}

typedef struct {
    unsigned count[256];
    size_t n;
    unsigned maxSym;
    size_t card;
} Stats;

static void stats_init(Stats* st, const uint8_t* src, size_t n)
{
    memset(st, 0, sizeof(*st));
    st->n = n;
    /* four partial tables, so that runs of one symbol do not serialize on
     * one counter */
    uint32_t part[4][256];
    memset(part, 0, sizeof(part));
    size_t i = 0;
    for (; i + 4 <= n; i += 4) {
        part[0][src[i]]++;
        part[1][src[i + 1]]++;
        part[2][src[i + 2]]++;
        part[3][src[i + 3]]++;
    }
    for (; i < n; i++) part[0][src[i]]++;
    for (int s = 0; s < 256; s++) st->count[s] = part[0][s] + part[1][s] + part[2][s] + part[3][s];
    for (int s = 0; s < 256; s++)
        if (st->count[s]) { st->card++; st->maxSym = (unsigned)s; }
}

static double stats_entropy(const Stats* st) { return calc_entropy(st->count, 255, st->n); }

/* DataStatsU8_estimateHuffmanSizeFast (data_stats.c:287-301) */
static size_t stats_huf_fast(const Stats* st)
{
    double e = stats_entropy(st);
    if (e > 7) return st->n;
    if (e < 1) e = 1;
    volatile double prod = e * (double)st->n;
    volatile double q = prod / 8;
    return (size_t)q;
}

static size_t stats_bitpacked(const Stats* st)
{
    if (!st->n) return 0;
    return (st->n * (size_t)ozo_nextpow2(st->maxSym + 1) + 7) / 8;
}

static size_t stats_flatpacked(const Stats* st)
{
    return (st->n * (size_t)ozo_nextpow2(st->card) + 7) / 8 + st->card;
}

/* ------------------------------------------------------------------ */
/* forward bit writer (src/openzl/fse/bitstream.h BIT_CStream): fields are
 * appended LSB-first; closing adds a 1 marker bit. */
typedef struct {
    uint8_t* buf;
    size_t cap, pos;
    uint64_t acc;
    unsigned nb;
} BW;

/* moves the whole bytes of the accumulator to the buffer: one 8-byte store
 * where it fits, else byte by byte up to the capacity */
static inline void bw_flush(BW* b)
{
    if (b->pos + 8 <= b->cap) {
        ozo_wr64(b->buf + b->pos, b->acc);
        unsigned const k = b->nb >> 3;
        b->pos += k;
        b->acc = k == 8 ? 0 : b->acc >> (8 * k);
        b->nb &= 7;
        return;
    }
    while (b->nb >= 8) {
        if (b->pos < b->cap) b->buf[b->pos] = (uint8_t)b->acc;
        b->pos++;
        b->acc >>= 8;
        b->nb -= 8;
    }
}
static inline void bw_add(BW* b, uint64_t v, unsigned nb)
{
    if (!nb) return;
    if (nb > 32) { /* two halves, low first */
        bw_add(b, v & 0xFFFFFFFFu, 32);
        bw_add(b, v >> 32, nb - 32);
        return;
    }
    v &= (1ull << nb) - 1;
    if (b->nb + nb > 64) bw_flush(b);
    b->acc |= v << b->nb;
    b->nb += nb;
}
static size_t bw_close(BW* b)
{
    bw_add(b, 1, 1);
    bw_flush(b);
    if (b->nb) {
        if (b->pos < b->cap) b->buf[b->pos] = (uint8_t)b->acc;
        b->pos++;
    }
    return b->pos <= b->cap ? b->pos : 0;
}

/* ------------------------------------------------------------------ */
/* FSE compression (src/openzl/fse/compress/fse_compress.c) */
static unsigned fse_min_tablelog(size_t srcSize, unsigned maxSV)
{
    unsigned a = (unsigned)ozo_highbit32((uint32_t)srcSize) + 1;
    unsigned b = (unsigned)ozo_highbit32(maxSV) + 2;
    return a < b ? a : b;
}

/* FSE_optimalTableLog_internal (fse_compress.c:379-396) */
static unsigned fse_optimal_tablelog(unsigned maxTL, size_t srcSize, unsigned maxSV, unsigned minus)
{
    unsigned maxBitsSrc = (unsigned)ozo_highbit32((uint32_t)(srcSize - 1)) - minus;
    unsigned tl = maxTL;
    unsigned minBits = fse_min_tablelog(srcSize, maxSV);
    if (tl == 0) tl = 11;
    if (maxBitsSrc < tl) tl = maxBitsSrc;
    if (minBits > tl) tl = minBits;
    if (tl < 5) tl = 5;
    if (tl > 12) tl = 12;
    return tl;
}

/* FSE_normalizeM2 (fse_compress.c:400-470) */
static int fse_normalize_m2(int16_t* norm, unsigned tl, const unsigned* count, size_t total, unsigned maxSV,
                            int16_t lowProb)
{
    int16_t const NYA = -2;
    unsigned distributed = 0;
    uint32_t const lowThreshold = (uint32_t)(total >> tl);
    uint32_t lowOne = (uint32_t)((total * 3) >> (tl + 1));
    for (unsigned s = 0; s <= maxSV; s++) {
        if (count[s] == 0) { norm[s] = 0; continue; }
        if (count[s] <= lowThreshold) { norm[s] = lowProb; distributed++; total -= count[s]; continue; }
        if (count[s] <= lowOne) { norm[s] = 1; distributed++; total -= count[s]; continue; }
        norm[s] = NYA;
    }
    uint32_t toDistribute = (1u << tl) - distributed;
    if (toDistribute == 0) return 0;
    if ((total / toDistribute) > lowOne) {
        lowOne = (uint32_t)((total * 3) / (toDistribute * 2));
        for (unsigned s = 0; s <= maxSV; s++) {
            if (norm[s] == NYA && count[s] <= lowOne) {
                norm[s] = 1;
                distributed++;
                total -= count[s];
            }
        }
        toDistribute = (1u << tl) - distributed;
    }
    if (distributed == maxSV + 1) {
        unsigned maxV = 0, maxC = 0;
        for (unsigned s = 0; s <= maxSV; s++)
            if (count[s] > maxC) { maxV = s; maxC = count[s]; }
        norm[maxV] = (int16_t)(norm[maxV] + (int16_t)toDistribute);
        return 0;
    }
    if (total == 0) {
        for (unsigned s = 0; toDistribute > 0; s = (s + 1) % (maxSV + 1))
            if (norm[s] > 0) { toDistribute--; norm[s]++; }
        return 0;
    }
    {
        uint64_t const vStepLog = 62 - tl;
        uint64_t const mid = (1ull << (vStepLog - 1)) - 1;
        uint64_t const rStep = (((uint64_t)1 << vStepLog) * toDistribute + mid) / (uint32_t)total;
        uint64_t tmpTotal = mid;
        for (unsigned s = 0; s <= maxSV; s++) {
            if (norm[s] == NYA) {
                uint64_t const end = tmpTotal + (count[s] * rStep);
                uint32_t const sStart = (uint32_t)(tmpTotal >> vStepLog);
                uint32_t const sEnd = (uint32_t)(end >> vStepLog);
                uint32_t const weight = sEnd - sStart;
                if (weight < 1) return -1;
                norm[s] = (int16_t)weight;
                tmpTotal = end;
            }
        }
    }
    return 0;
}

/* FSE_normalizeCount (fse_compress.c:472-520) */
static int fse_normalize(int16_t* norm, unsigned tl, const unsigned* count, size_t total, unsigned maxSV,
                         int useLowProb)
{
    static const uint32_t rtb[] = { 0, 473195, 504333, 520860, 550000, 700000, 750000, 830000 };
    int16_t const lowProb = useLowProb ? -1 : 1;
    uint64_t const scale = 62 - tl;
    uint64_t const step = ((uint64_t)1 << 62) / (uint32_t)total;
    uint64_t const vStep = 1ull << (scale - 20);
    int still = 1 << tl;
    unsigned largest = 0;
    int16_t largestP = 0;
    uint32_t const lowThreshold = (uint32_t)(total >> tl);
    for (unsigned s = 0; s <= maxSV; s++) {
        if (count[s] == total) return 0;
        if (count[s] == 0) { norm[s] = 0; continue; }
        if (count[s] <= lowThreshold) {
            norm[s] = lowProb;
            still--;
        } else {
            int16_t proba = (int16_t)((count[s] * step) >> scale);
            if (proba < 8) {
                uint64_t const restToBeat = vStep * rtb[proba];
                proba = (int16_t)(proba + ((count[s] * step) - ((uint64_t)proba << scale) > restToBeat));
            }
            if (proba > largestP) { largestP = proba; largest = s; }
            norm[s] = proba;
            still -= proba;
        }
    }
    if (-still >= (norm[largest] >> 1)) return fse_normalize_m2(norm, tl, count, total, maxSV, lowProb);
    norm[largest] = (int16_t)(norm[largest] + (int16_t)still);
    return 0;
}

/* FSE_buildCTable_wksp (fse_compress.c:69-207): state table sorted by
 * symbol and the per-symbol transform (deltaNbBits, deltaFindState). */
typedef struct {
    unsigned tl;
    uint16_t state[4096];
    uint32_t deltaNbBits[256];
    int32_t deltaFindState[256];
} FseC;

static void fse_build_ctable(FseC* ct, const int16_t* norm, unsigned maxSV, unsigned tl)
{
    uint32_t const size = 1u << tl, mask = size - 1, step = (size >> 1) + (size >> 3) + 3;
    uint16_t cumul[258];
    uint8_t sym[4096];
    uint32_t high = size - 1;
    ct->tl = tl;
    cumul[0] = 0;
    for (unsigned u = 1; u <= maxSV + 1; u++) {
        if (norm[u - 1] == -1) {
            cumul[u] = (uint16_t)(cumul[u - 1] + 1);
            sym[high--] = (uint8_t)(u - 1);
        } else {
            cumul[u] = (uint16_t)(cumul[u - 1] + (uint16_t)norm[u - 1]);
        }
    }
    cumul[maxSV + 1] = (uint16_t)(size + 1);
    uint32_t pos = 0;
    for (unsigned s = 0; s <= maxSV; s++) {
        for (int i = 0; i < norm[s]; i++) {
            sym[pos] = (uint8_t)s;
            do { pos = (pos + step) & mask; } while (pos > high);
        }
    }
    for (uint32_t u = 0; u < size; u++) ct->state[cumul[sym[u]]++] = (uint16_t)(size + u);
    unsigned total = 0;
    for (unsigned s = 0; s <= maxSV; s++) {
        switch (norm[s]) {
            case 0: ct->deltaNbBits[s] = ((tl + 1) << 16) - (1u << tl); break;
            case -1:
            case 1:
                ct->deltaNbBits[s] = (tl << 16) - (1u << tl);
                ct->deltaFindState[s] = (int)(total - 1);
                total++;
                break;
            default: {
                uint32_t const maxBitsOut = tl - (unsigned)ozo_highbit32((uint32_t)norm[s] - 1);
                uint32_t const minStatePlus = (uint32_t)norm[s] << maxBitsOut;
                ct->deltaNbBits[s] = (maxBitsOut << 16) - minStatePlus;
                ct->deltaFindState[s] = (int)(total - (unsigned)norm[s]);
                total += (unsigned)norm[s];
            }
        }
    }
}

typedef struct {
    uint64_t value;
} FseState;

static void fse_init_state2(FseState* st, const FseC* ct, unsigned symbol)
{
    uint32_t const nbBitsOut = (ct->deltaNbBits[symbol] + (1 << 15)) >> 16;
    uint32_t v = (nbBitsOut << 16) - ct->deltaNbBits[symbol];
    st->value = ct->state[(v >> nbBitsOut) + ct->deltaFindState[symbol]];
}

static void fse_encode_symbol(BW* b, FseState* st, const FseC* ct, unsigned symbol)
{
    uint32_t const nbBitsOut = (uint32_t)((st->value + ct->deltaNbBits[symbol]) >> 16);
    bw_add(b, st->value, nbBitsOut);
    st->value = ct->state[(st->value >> nbBitsOut) + ct->deltaFindState[symbol]];
}

/* FSE_compress_usingCTable_generic (fse_compress.c:607-658) */
static size_t fse_compress(uint8_t* dst, size_t cap, const uint8_t* src, size_t n, const FseC* ct,
                           unsigned nbStates)
{
    if (n <= nbStates) return 0;
    BW b = { dst, cap, 0, 0, 0 };
    FseState st[4];
    const uint8_t* ip = src + n;
    size_t s = nbStates - (n % nbStates);
    for (unsigned i = 0; i < nbStates; i++) fse_init_state2(&st[(s++) % nbStates], ct, *--ip);
    for (size_t i = 0; i < n % nbStates; i++) fse_encode_symbol(&b, &st[(s++) % nbStates], ct, *--ip);
    /* ip - src is a multiple of nbStates now: rounds of one symbol per
     * state, state 0 first. A field has at most 12 bits, so a round appends
     * at most 48 bits after one flush check. */
#define OZO_FSE_ENC(v)                                                                  \
    do {                                                                                \
        unsigned const y_ = *--ip;                                                      \
        uint32_t const nb_ = (uint32_t)(((v) + ct->deltaNbBits[y_]) >> 16);             \
        b.acc |= ((v) & ((1ull << nb_) - 1)) << b.nb;                                   \
        b.nb += nb_;                                                                    \
        (v) = ct->state[((v) >> nb_) + ct->deltaFindState[y_]];                         \
    } while (0)
    uint64_t v0 = st[0].value, v1 = st[1].value;
    if (nbStates == 4) {
        uint64_t v2 = st[2].value, v3 = st[3].value;
        while (ip > src) {
            if (b.nb > 16) bw_flush(&b);
            OZO_FSE_ENC(v0);
            OZO_FSE_ENC(v1);
            OZO_FSE_ENC(v2);
            OZO_FSE_ENC(v3);
        }
        st[2].value = v2;
        st[3].value = v3;
    } else {
        while (ip > src) {
            if (b.nb > 40) bw_flush(&b);
            OZO_FSE_ENC(v0);
            OZO_FSE_ENC(v1);
        }
    }
#undef OZO_FSE_ENC
    st[0].value = v0;
    st[1].value = v1;
    for (unsigned i = 0; i < nbStates; i++) bw_add(&b, st[i].value, ct->tl);
    return bw_close(&b);
}

/* FSE_writeNCount_generic (fse_compress.c:226-338) */
static size_t fse_write_ncount(uint8_t* out, const int16_t* norm, unsigned maxSV, unsigned tl)
{
    size_t op = 0;
    uint32_t bitStream = 0;
    int bitCount = 0;
    int const tableSize = 1 << tl;
    int remaining = tableSize + 1, threshold = tableSize, nbBits = (int)tl + 1;
    unsigned symbol = 0;
    unsigned const alphabet = maxSV + 1;
    int previousIs0 = 0;
    bitStream += (tl - 5) << bitCount;
    bitCount += 4;
    while (symbol < alphabet && remaining > 1) {
        if (previousIs0) {
            unsigned start = symbol;
            while (symbol < alphabet && !norm[symbol]) symbol++;
            if (symbol == alphabet) break;
            while (symbol >= start + 24) {
                start += 24;
                bitStream += 0xFFFFu << bitCount;
                out[op] = (uint8_t)bitStream;
                out[op + 1] = (uint8_t)(bitStream >> 8);
                op += 2;
                bitStream >>= 16;
            }
            while (symbol >= start + 3) {
                start += 3;
                bitStream += 3u << bitCount;
                bitCount += 2;
            }
            bitStream += (symbol - start) << bitCount;
            bitCount += 2;
            if (bitCount > 16) {
                out[op] = (uint8_t)bitStream;
                out[op + 1] = (uint8_t)(bitStream >> 8);
                op += 2;
                bitStream >>= 16;
                bitCount -= 16;
            }
        }
        {
            int count = norm[symbol++];
            int const max = (2 * threshold - 1) - remaining;
            remaining -= count < 0 ? -count : count;
            count++;
            if (count >= threshold) count += max;
            bitStream += (uint32_t)count << bitCount;
            bitCount += nbBits;
            bitCount -= (count < max);
            previousIs0 = (count == 1);
            while (remaining < threshold) { nbBits--; threshold >>= 1; }
        }
        if (bitCount > 16) {
            out[op] = (uint8_t)bitStream;
            out[op + 1] = (uint8_t)(bitStream >> 8);
            op += 2;
            bitStream >>= 16;
            bitCount -= 16;
        }
    }
    out[op] = (uint8_t)bitStream;
    out[op + 1] = (uint8_t)(bitStream >> 8);
    op += (size_t)((bitCount + 7) / 8);
    return op;
}

/* ------------------------------------------------------------------ */
/* Huffman compression (src/openzl/fse/compress/huf_compress.c) */
typedef struct {
    uint32_t count;
    uint16_t parent;
    uint8_t byte;
    uint8_t nbBits;
} HNode;

/* HUF_getIndex (huf_compress.c:484-509): the distinct-count cutoff is
 * 158 + highbit32(158) = 165 by the reference's macro arithmetic (its
 * comment says 166), and HUF_sort quicksorts rank buckets from 165 on, rank
 * r holding index r - 1: the bucket of count 164 is sorted too. */
static uint32_t huf_index(uint32_t c) { return c < 165 ? c : (uint32_t)ozo_highbit32(c) + 158; }

static void huf_insertion(HNode* a, int low, int high)
{
    int const size = high - low + 1;
    a += low;
    for (int i = 1; i < size; i++) {
        HNode const key = a[i];
        int j = i - 1;
        while (j >= 0 && a[j].count < key.count) { a[j + 1] = a[j]; j--; }
        a[j + 1] = key;
    }
}

static int huf_partition(HNode* a, int low, int high)
{
    uint32_t const pivot = a[high].count;
    int i = low - 1;
    for (int j = low; j < high; j++)
        if (a[j].count > pivot) {
            i++;
            HNode t = a[i]; a[i] = a[j]; a[j] = t;
        }
    HNode t = a[i + 1]; a[i + 1] = a[high]; a[high] = t;
    return i + 1;
}

static void huf_quicksort(HNode* a, int low, int high)
{
    if (high - low < 8) { huf_insertion(a, low, high); return; }
    while (low < high) {
        int const idx = huf_partition(a, low, high);
        if (idx - low < high - idx) { huf_quicksort(a, low, idx - 1); low = idx + 1; }
        else { huf_quicksort(a, idx + 1, high); high = idx - 1; }
    }
}

/* HUF_sort (huf_compress.c:586-631): bucket sort by count, quicksort in the
 * logarithmic buckets. */
static void huf_sort(HNode* node, const unsigned* count, unsigned maxSV)
{
    struct { uint16_t base, curr; } rank[192];
    memset(rank, 0, sizeof(rank));
    for (unsigned n = 0; n <= maxSV; n++) rank[huf_index(count[n])].base++;
    for (int n = 191; n > 0; n--) {
        rank[n - 1].base = (uint16_t)(rank[n - 1].base + rank[n].base);
        rank[n - 1].curr = rank[n - 1].base;
    }
    for (unsigned n = 0; n <= maxSV; n++) {
        uint32_t const r = huf_index(count[n]) + 1;
        uint32_t const pos = rank[r].curr++;
        node[pos].count = count[n];
        node[pos].byte = (uint8_t)n;
    }
    for (int n = 165; n < 191; n++) {
        int const bs = rank[n].curr - rank[n].base;
        if (bs > 1) huf_quicksort(node + rank[n].base, 0, bs - 1);
    }
}

/* HUF_setMaxHeight (huf_compress.c:352-470) */
static uint32_t huf_set_max_height(HNode* node, uint32_t last, uint32_t target)
{
    uint32_t const largest = node[last].nbBits;
    if (largest <= target) return largest;
    int totalCost = 0;
    int const baseCost = 1 << (largest - target);
    int n = (int)last;
    while (node[n].nbBits > target) {
        totalCost += baseCost - (1 << (largest - node[n].nbBits));
        node[n].nbBits = (uint8_t)target;
        n--;
    }
    while (node[n].nbBits == target) --n;
    totalCost >>= (largest - target);
    uint32_t const noSym = 0xF0F0F0F0u;
    uint32_t rankLast[14];
    for (int i = 0; i < 14; i++) rankLast[i] = noSym;
    {
        uint32_t cur = target;
        for (int pos = n; pos >= 0; pos--) {
            if (node[pos].nbBits >= cur) continue;
            cur = node[pos].nbBits;
            rankLast[target - cur] = (uint32_t)pos;
        }
    }
    while (totalCost > 0) {
        uint32_t nb = (uint32_t)ozo_highbit32((uint32_t)totalCost) + 1;
        for (; nb > 1; nb--) {
            uint32_t const highPos = rankLast[nb];
            uint32_t const lowPos = rankLast[nb - 1];
            if (highPos == noSym) continue;
            if (lowPos == noSym) break;
            if (node[highPos].count <= 2 * node[lowPos].count) break;
        }
        while (nb <= 12 && rankLast[nb] == noSym) nb++;
        totalCost -= 1 << (nb - 1);
        node[rankLast[nb]].nbBits++;
        if (rankLast[nb - 1] == noSym) rankLast[nb - 1] = rankLast[nb];
        if (rankLast[nb] == 0) {
            rankLast[nb] = noSym;
        } else {
            rankLast[nb]--;
            if (node[rankLast[nb]].nbBits != target - nb) rankLast[nb] = noSym;
        }
    }
    while (totalCost < 0) {
        if (rankLast[1] == noSym) {
            while (node[n].nbBits == target) n--;
            node[n + 1].nbBits--;
            rankLast[1] = (uint32_t)(n + 1);
            totalCost++;
            continue;
        }
        node[rankLast[1] + 1].nbBits--;
        rankLast[1]++;
        totalCost++;
    }
    return target;
}

typedef struct {
    uint8_t nbBits[256];
    uint16_t value[256];
    unsigned maxNbBits;
} HufC;

/* HUF_buildCTable_wksp (huf_compress.c:650-760) */
static unsigned huf_build_ctable(HufC* ct, const unsigned* count, unsigned maxSV, unsigned maxNbBits)
{
    HNode all[2 * 256 + 2];
    memset(all, 0, sizeof(all));
    HNode* node = all + 1;
    huf_sort(node, count, maxSV);
    /* tree */
    int const startNode = 256;
    int nonNull = (int)maxSV;
    while (node[nonNull].count == 0) nonNull--;
    int lowS = nonNull, nodeNb = startNode;
    int const nodeRoot = nodeNb + lowS - 1;
    int lowN = nodeNb;
    node[nodeNb].count = node[lowS].count + node[lowS - 1].count;
    node[lowS].parent = node[lowS - 1].parent = (uint16_t)nodeNb;
    nodeNb++;
    lowS -= 2;
    for (int n = nodeNb; n <= nodeRoot; n++) node[n].count = 1u << 30;
    all[0].count = 1u << 31;
    while (nodeNb <= nodeRoot) {
        int const n1 = node[lowS].count < node[lowN].count ? lowS-- : lowN++;
        int const n2 = node[lowS].count < node[lowN].count ? lowS-- : lowN++;
        node[nodeNb].count = node[n1].count + node[n2].count;
        node[n1].parent = node[n2].parent = (uint16_t)nodeNb;
        nodeNb++;
    }
    node[nodeRoot].nbBits = 0;
    for (int n = nodeRoot - 1; n >= startNode; n--) node[n].nbBits = (uint8_t)(node[node[n].parent].nbBits + 1);
    for (int n = 0; n <= nonNull; n++) node[n].nbBits = (uint8_t)(node[node[n].parent].nbBits + 1);
    maxNbBits = huf_set_max_height(node, (uint32_t)nonNull, maxNbBits);
    /* codes */
    uint16_t nbPerRank[13] = { 0 }, valPerRank[13] = { 0 };
    for (int n = 0; n <= nonNull; n++) nbPerRank[node[n].nbBits]++;
    {
        uint16_t min = 0;
        for (int n = (int)maxNbBits; n > 0; n--) {
            valPerRank[n] = min;
            min = (uint16_t)(min + nbPerRank[n]);
            min >>= 1;
        }
    }
    memset(ct, 0, sizeof(*ct));
    for (unsigned n = 0; n <= maxSV; n++) ct->nbBits[node[n].byte] = node[n].nbBits;
    for (unsigned n = 0; n <= maxSV; n++) ct->value[n] = valPerRank[ct->nbBits[n]]++;
    ct->maxNbBits = maxNbBits;
    return maxNbBits;
}

/* HUF 1X stream: symbols from last to first, codes appended LSB-first. */
static size_t huf_compress1x(uint8_t* dst, size_t cap, const uint8_t* src, size_t n, const HufC* ct)
{
    BW b = { dst, cap, 0, 0, 0 };
    size_t i = n;
    /* codes of at most 12 bits (values hold no bits above their length):
     * four per flush check */
    for (; i >= 4; i -= 4) {
        if (b.nb > 16) bw_flush(&b);
        for (int k = 1; k <= 4; k++) {
            unsigned const y = src[i - (size_t)k];
            b.acc |= (uint64_t)ct->value[y] << b.nb;
            b.nb += ct->nbBits[y];
        }
    }
    for (; i > 0; i--) bw_add(&b, ct->value[src[i - 1]], ct->nbBits[src[i - 1]]);
    return bw_close(&b);
}

/* HUF_compress4X_usingCTable_internal (huf_compress.c:1139-1190) */
static size_t huf_compress4x(uint8_t* dst, size_t cap, const uint8_t* src, size_t n, const HufC* ct)
{
    size_t const seg = (n + 3) / 4;
    if (n < 12 || cap < 6 + 4) return 0;
    size_t op = 6;
    for (int k = 0; k < 4; k++) {
        size_t const start = seg * (size_t)k;
        size_t const len = k < 3 ? seg : n - 3 * seg;
        size_t const c = huf_compress1x(dst + op, cap - op, src + start, len, ct);
        if (c == 0 || c > 65535) return 0;
        if (k < 3) ozo_wr16(dst + 2 * k, (uint16_t)c);
        op += c;
    }
    return op;
}

/* ------------------------------------------------------------------ */
/* 16-bit-symbol Huffman (src/openzl/codecs/entropy/encode_huffman_kernel.c) */
typedef struct {
    uint32_t count, parent;
    uint16_t symbol, nbBits;
} LNode;

/* ZS_largeHuffmanSort (encode_huffman_kernel.c:153-229): counts in
 * decreasing order. The reference's partition by highest set bit, recursing
 * into each partition on the remaining bits, is stable, so equal counts stay
 * in symbol order. */
static int lnode_cmp(const void* a, const void* b)
{
    const LNode* x = (const LNode*)a;
    const LNode* y = (const LNode*)b;
    if (x->count != y->count) return x->count > y->count ? -1 : 1;
    return (int)x->symbol - (int)y->symbol;
}

/* ZS_largeHuffmanBuildTree (encode_huffman_kernel.c:231-290); node[-1] is the
 * sentinel slot. */
static int lhuf_build_tree(LNode* node, int maxSV)
{
    int nonNull = maxSV;
    while (node[nonNull].count == 0) nonNull--;
    int const startNode = maxSV + 1;
    int nodeNb = startNode, lowS = nonNull, lowN = nodeNb;
    int const nodeRoot = nodeNb + lowS - 1;
    node[nodeNb].count = node[lowS].count + node[lowS - 1].count;
    node[lowS].parent = node[lowS - 1].parent = (uint32_t)nodeNb;
    nodeNb++;
    lowS -= 2;
    for (int n = nodeNb; n <= nodeRoot; n++) node[n].count = 1u << 30;
    node[-1].count = 1u << 31;
    for (; nodeNb <= nodeRoot; nodeNb++) {
        int const n1 = node[lowS].count < node[lowN].count ? lowS-- : lowN++;
        int const n2 = node[lowS].count < node[lowN].count ? lowS-- : lowN++;
        node[nodeNb].count = node[n1].count + node[n2].count;
        node[n1].parent = node[n2].parent = (uint32_t)nodeNb;
    }
    node[nodeRoot].nbBits = 0;
    for (int n = nodeRoot - 1; n >= startNode; n--) node[n].nbBits = (uint16_t)(node[node[n].parent].nbBits + 1);
    for (int n = 0; n <= nonNull; n++) node[n].nbBits = (uint16_t)(node[node[n].parent].nbBits + 1);
    return nonNull;
}

/* ZS_largeHuffmanSetMaxHeight (encode_huffman_kernel.c:34-151) */
static int lhuf_set_max_height(LNode* node, int last, int maxNbBits)
{
    int const largest = node[last].nbBits;
    if (largest <= maxNbBits) return largest;
    int totalCost = 0;
    int const baseCost = 1 << (largest - maxNbBits);
    int n;
    for (n = last; node[n].nbBits > maxNbBits; --n) {
        totalCost += baseCost - (1 << (largest - node[n].nbBits));
        node[n].nbBits = (uint16_t)maxNbBits;
    }
    while (node[n].nbBits == maxNbBits) --n;
    totalCost >>= (largest - maxNbBits);
    uint32_t const noSym = 0xF0F0F0F0u;
    uint32_t rankLast[22];
    for (int i = 0; i < 22; i++) rankLast[i] = noSym;
    {
        int cur = maxNbBits;
        for (int pos = n; pos >= 0; pos--) {
            if (node[pos].nbBits >= cur) continue;
            cur = node[pos].nbBits;
            rankLast[maxNbBits - cur] = (uint32_t)pos;
        }
    }
    while (totalCost > 0) {
        int nb = ozo_highbit32((uint32_t)totalCost) + 1;
        while (nb > 1 && rankLast[nb] == noSym) --nb;
        for (; nb > 1; nb--) {
            uint32_t const highPos = rankLast[nb], lowPos = rankLast[nb - 1];
            if (highPos == noSym || lowPos == noSym) break;
            if (node[highPos].count <= 2 * node[lowPos].count) break;
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
            rankLast[1] = (uint32_t)(n + 1);
            totalCost++;
            continue;
        }
        node[rankLast[1] + 1].nbBits--;
        rankLast[1]++;
        totalCost++;
    }
    return maxNbBits;
}

/* ZS_largeHuffmanBuildCTable with maxNbBits 0 (encode_huffman_kernel.c:292-374):
 * code lengths and canonical codes per symbol (16-bit code arithmetic, as in
 * the reference). Returns the table log, or -1. */
static int lhuf_build_ctable(uint16_t* code, uint16_t* nbBits, const unsigned* count, unsigned maxSV)
{
    int maxNbBits = 20;
    int const bound = ozo_nextpow2((uint64_t)maxSV + 1);
    if (bound + 3 < maxNbBits) maxNbBits = bound + 3;
    LNode* all = (LNode*)calloc(2 * (size_t)maxSV + 3, sizeof(LNode));
    LNode* node = all + 1;
    for (unsigned s = 0; s <= maxSV; s++) {
        node[s].count = count[s];
        node[s].symbol = (uint16_t)s;
    }
    qsort(node, (size_t)maxSV + 1, sizeof(LNode), lnode_cmp);
    int const nonNull = lhuf_build_tree(node, (int)maxSV);
    maxNbBits = lhuf_set_max_height(node, nonNull, maxNbBits);
    if (maxNbBits < 0 || maxNbBits > 20) { free(all); return -1; }
    uint16_t nbPerRank[21] = { 0 }, valPerRank[21] = { 0 };
    for (int k = 0; k <= nonNull; k++) nbPerRank[node[k].nbBits]++;
    {
        uint16_t min = 0;
        for (int k = maxNbBits; k > 0; k--) {
            valPerRank[k] = min;
            min = (uint16_t)(min + nbPerRank[k]);
            min >>= 1;
        }
    }
    for (unsigned k = 0; k <= maxSV; k++) nbBits[node[k].symbol] = node[k].nbBits;
    for (unsigned s = 0; s <= maxSV; s++) code[s] = valPerRank[nbBits[s]]++;
    free(all);
    return maxNbBits;
}

/* ZS_largeHuffmanEncodeUsingCTable (encode_huffman_kernel.c:413-488): the
 * symbol count and the stream size as LE32, then the symbols from last to
 * first, codes appended LSB-first, closed by a 1 bit. The bit writer gives up
 * (0) once its output reaches 8 bytes before the end of the capacity. */
static size_t lhuf_stream(uint8_t* dst, size_t cap, const uint8_t* src, size_t n, const uint16_t* code,
                          const uint16_t* nbBits)
{
    if (cap < 8) return 0;
    ozo_wr32(dst, (uint32_t)n);
    size_t const bcap = cap - 8;
    if (bcap <= 8) return 0;
    BW b = { dst + 8, bcap, 0, 0, 0 };
    for (size_t i = n; i > 0; i--) {
        uint16_t const s = ozo_rd16(src + 2 * (i - 1));
        bw_add(&b, code[s], nbBits[s]);
    }
    bw_add(&b, 1, 1);
    bw_flush(&b);
    size_t const full = b.pos;
    if (full >= bcap - 8) return 0;
    size_t const sz = full + (b.nb > 0);
    if (b.nb) dst[8 + full] = (uint8_t)b.acc;
    ozo_wr32(dst + 4, (uint32_t)sz);
    return 8 + sz;
}

/* ------------------------------------------------------------------ */
/* engine: graph runs */
static int run_successor(ECtx* c, int g, int sid, const void* arg);

typedef struct {
    int g;
    int sid;
    const void* arg;
} Succ;

typedef struct {
    Succ* v;
    size_t n, cap;
} SuccList;

static void succ_add(SuccList* l, int g, int sid, const void* arg)
{
    if (l->n == l->cap) {
        l->cap = l->cap ? 2 * l->cap : 16;
        l->v = (Succ*)realloc(l->v, l->cap * sizeof(Succ));
    }
    l->v[l->n].g = g;
    l->v[l->n].sid = sid;
    l->v[l->n].arg = arg;
    l->n++;
}

static int succ_cmp(const void* a, const void* b)
{
    return ((const Succ*)a)->sid - ((const Succ*)b)->sid;
}

/* Successors run in the order their edges were created, which is stream-id
 * order within a graph (src/openzl/compress/cctx.c:660-690). */
static int run_succs(ECtx* c, SuccList* l)
{
    int rc = 0;
    if (l->n > 1) qsort(l->v, l->n, sizeof(Succ), succ_cmp);
    for (size_t i = 0; i < l->n && !rc; i++) rc = run_successor(c, l->v[i].g, l->v[i].sid, l->v[i].arg);
    free(l->v);
    return rc;
}

/* conversion nodes (encode_conversion_binding.c) */
static int node_conv_num_to_serial(ECtx* c, int in)
{
    ENode* nd = new_node(c, TR_CONV_NUM_TO_SERIAL_LE, in, 1);
    nd->hdr[0] = (uint8_t)ozo_nextpow2(S(in)->w);
    nd->hsz = 1;
    int o = new_stream(c, OZO_TYPE_SERIAL, 1, S(in)->n * S(in)->w, S(in)->data);
    nd->nbOut = 1;
    return o;
}
static int node_conv_struct_to_serial(ECtx* c, int in)
{
    ENode* nd = new_node(c, TR_CONV_STRUCT_TO_SERIAL, in, 1);
    nd->hsz = ozo_varint_enc(nd->hdr, S(in)->w);
    int o = new_stream(c, OZO_TYPE_SERIAL, 1, S(in)->n * S(in)->w, S(in)->data);
    nd->nbOut = 1;
    return o;
}
static int node_conv_num_to_struct(ECtx* c, int in)
{
    ENode* nd = new_node(c, TR_CONV_NUM_TO_STRUCT_LE, in, 1);
    int o = new_stream(c, OZO_TYPE_STRUCT, S(in)->w, S(in)->n, S(in)->data);
    nd->nbOut = 1;
    return o;
}

/* ZL_NODE_INTERPRET_TOKEN_AS_LE: struct tokens read as little-endian
 * numbers, no codec header (encode_conversion_binding.c:179-189) */
static int node_conv_struct_to_num(ECtx* c, int in)
{
    ENode* nd = new_node(c, TR_CONV_STRUCT_TO_NUM_LE, in, 1);
    int o = new_stream(c, OZO_TYPE_NUMERIC, S(in)->w, S(in)->n, S(in)->data);
    nd->nbOut = 1;
    return o;
}

/* implicit conversion towards a graph's accepted types (implicit_conversion.c:18-34) */
static int convert_for(ECtx* c, int sid, int mask)
{
    int const t = S(sid)->type;
    if (t & mask) return sid;
    if ((t & OZO_TYPE_NUMERIC) && (mask & OZO_TYPE_STRUCT)) return node_conv_num_to_struct(c, sid);
    if ((t & OZO_TYPE_STRUCT) && (mask & OZO_TYPE_SERIAL)) return node_conv_struct_to_serial(c, sid);
    if ((t & OZO_TYPE_NUMERIC) && (mask & OZO_TYPE_SERIAL)) return node_conv_num_to_serial(c, sid);
    c->err = OZO_ERR_UNSUPPORTED;
    return sid;
}

/* codecs: each creates its node and output streams, returns first output */
static int node_delta(ECtx* c, int in)
{
    EStream* I = S(in);
    size_t const w = I->w, n = I->n;
    ENode* nd = new_node(c, TR_DELTA_INT, in, 1);
    int o = new_stream(c, OZO_TYPE_NUMERIC, w, n ? n - 1 : 0, NULL);
    nd->nbOut = 1;
    I = S(in);
    if (n) {
        memcpy(nd->hdr, I->data, w);
        nd->hsz = w;
        const uint8_t* const x = I->data;
        uint8_t* const d = S(o)->data;
#define OZO_DELTA_ENC(T)                                  \
    for (size_t i = 1; i < n; i++) {                      \
        T a, b;                                           \
        memcpy(&a, x + (i - 1) * sizeof(T), sizeof(T));   \
        memcpy(&b, x + i * sizeof(T), sizeof(T));         \
        b = (T)(b - a);                                   \
        memcpy(d + (i - 1) * sizeof(T), &b, sizeof(T));   \
    }
        switch (w) {
            case 1: OZO_DELTA_ENC(uint8_t) break;
            case 2: OZO_DELTA_ENC(uint16_t) break;
            case 4: OZO_DELTA_ENC(uint32_t) break;
            case 8: OZO_DELTA_ENC(uint64_t) break;
            default: {
                uint64_t const m = (1ull << (8 * w)) - 1;
                for (size_t i = 1; i < n; i++)
                    wr(d + (i - 1) * w, (rd(x + i * w, w) - rd(x + (i - 1) * w, w)) & m, w);
            }
        }
#undef OZO_DELTA_ENC
    }
    return o;
}

static int node_zigzag(ECtx* c, int in)
{
    size_t const w = S(in)->w, n = S(in)->n;
    ENode* nd = new_node(c, TR_ZIGZAG, in, 1);
    int o = new_stream(c, OZO_TYPE_NUMERIC, w, n, NULL);
    nd->nbOut = 1;
    uint64_t const m = w == 8 ? ~0ull : ((1ull << (8 * w)) - 1);
    unsigned const sh = (unsigned)(8 * w - 1);
    for (size_t i = 0; i < n; i++) {
        uint64_t v = rd(S(in)->data + i * w, w);
        uint64_t sign = (v >> sh) & 1;
        wr(S(o)->data + i * w, ((v << 1) ^ (0 - sign)) & m, w);
    }
    return o;
}

/* EI_bitpack_typed (encode_bitpack_binding.c:93-147) */
static int node_bitpack(ECtx* c, int in, unsigned trid)
{
    size_t const w = S(in)->w, n = S(in)->n;
    uint64_t mx = 0;
    const uint8_t* const x = S(in)->data;
#define OZO_MAX_W(T)                                  \
    for (size_t i = 0; i < n; i++) {                  \
        T v;                                          \
        memcpy(&v, x + i * sizeof(T), sizeof(T));     \
        if (v > mx) mx = v;                           \
    }
    switch (w) {
        case 1: OZO_MAX_W(uint8_t) break;
        case 2: OZO_MAX_W(uint16_t) break;
        case 4: OZO_MAX_W(uint32_t) break;
        case 8: OZO_MAX_W(uint64_t) break;
        default:
            for (size_t i = 0; i < n; i++) {
                uint64_t v = rd(x + i * w, w);
                if (v > mx) mx = v;
            }
    }
#undef OZO_MAX_W
    int const nbBits = 1 + (mx ? ozo_highbit64(mx) : 0);
    size_t const dstSize = (n * (size_t)nbBits + 7) / 8;
    ENode* nd = new_node(c, trid, in, 1);
    int o = new_stream(c, OZO_TYPE_SERIAL, 1, dstSize, NULL);
    nd->nbOut = 1;
    uint8_t* d = S(o)->data;
    memset(d, 0, dstSize + 8);
    /* LSB-first: fields go into an accumulator above the bits not yet
     * written; whole words are flushed. Fields of at most 32 bits use a
     * 64-bit accumulator (32-bit flushes), wider ones a 128-bit one. */
    uint8_t* q = d;
    if (nbBits <= 32) {
        uint64_t acc = 0;
        unsigned nacc = 0;
#define OZO_PACK32(READ)                                      for (size_t i = 0; i < n; i++) {                              acc |= (uint64_t)(READ) << nacc;                          nacc += (unsigned)nbBits;                                 if (nacc >= 32) {                                             ozo_wr32(q, (uint32_t)acc);                               q += 4;                                                   acc >>= 32;                                               nacc -= 32;                                           }                                                     }
        switch (w) {
            case 1: OZO_PACK32(x[i]) break;
            case 2: OZO_PACK32(ozo_rd16(x + 2 * i)) break;
            case 4: OZO_PACK32(ozo_rd32(x + 4 * i)) break;
            default: OZO_PACK32(rd(x + i * w, w)) break;
        }
#undef OZO_PACK32
        for (; nacc > 0; nacc = nacc > 8 ? nacc - 8 : 0) {
            *q++ = (uint8_t)acc;
            acc >>= 8;
        }
    } else {
        unsigned __int128 acc = 0;
        unsigned nacc = 0;
        for (size_t i = 0; i < n; i++) {
            uint64_t const v = rd(x + i * w, w);
            acc |= (unsigned __int128)v << nacc;
            nacc += (unsigned)nbBits;
            if (nacc >= 64) {
                ozo_wr64(q, (uint64_t)acc);
                q += 8;
                acc >>= 64;
                nacc -= 64;
            }
        }
        for (; nacc > 0; nacc = nacc > 8 ? nacc - 8 : 0) {
            *q++ = (uint8_t)acc;
            acc >>= 8;
        }
    }
    size_t const maxN = dstSize * 8 / (size_t)nbBits;
    static const uint8_t lg[9] = { 0, 0, 1, 0, 2, 0, 0, 0, 3 };
    nd->hdr[0] = (uint8_t)((lg[w] << 6) | (nbBits - 1));
    nd->hsz = 1;
    if (maxN > n) {
        nd->hdr[1] = (uint8_t)(maxN - n);
        nd->hsz = 2;
    }
    return o;
}

/* EI_transpose_split: W serial planes */
static int node_tsplit(ECtx* c, int in)
{
    size_t const W = S(in)->w, n = S(in)->n;
    ENode* nd = new_node(c, TR_TRANSPOSE_SPLIT, in, 0);
    int first = -1;
    uint8_t* planes[8];
    for (size_t b = 0; b < W; b++) {
        int o = new_stream(c, OZO_TYPE_SERIAL, 1, n, NULL);
        if (first < 0) first = o;
        if (b < 8) planes[b] = S(o)->data;
    }
    const uint8_t* const x = S(in)->data;
    if (W == 2 || W == 4 || W == 8) { /* element-major: one pass over the input */
        for (size_t e = 0; e < n; e++) {
            uint64_t const v = rd(x + e * W, W);
            for (size_t b = 0; b < W; b++) planes[b][e] = (uint8_t)(v >> (8 * b));
        }
    } else {
        for (size_t b = 0; b < W; b++) {
            uint8_t* const pl = S(first + (int)b)->data;
            for (size_t e = 0; e < n; e++) pl[e] = x[e * W + b];
        }
    }
    nd->nbOut = (int)W;
    return first;
}

/* EI_splitN over fixed chunk sizes (encode_splitN_binding.c:105-160); the
 * transform follows the stream type (getSplitNNodeID,
 * encode_splitN_binding.c:163-176) */
static int node_splitn(ECtx* c, int in, const size_t* sizes, size_t nb)
{
    int const t = S(in)->type;
    ENode* nd = new_node(c, t == OZO_TYPE_STRUCT ? TR_SPLITN_STRUCT : t == OZO_TYPE_NUMERIC ? TR_SPLITN_NUM : TR_SPLITN,
                         in, 0);
    size_t pos = 0;
    int first = -1;
    for (size_t k = 0; k < nb; k++) {
        int o = new_stream(c, S(in)->type, S(in)->w, sizes[k], S(in)->data + pos * S(in)->w);
        if (first < 0) first = o;
        pos += sizes[k];
    }
    nd->nbOut = (int)nb;
    return first;
}

/* EI_constant_typed (encode_constant_binding.c:13-44): a serial or struct
 * input whose elements are all equal (else node_invalid_input); the first
 * element is the output, the element count the codec header. */
static int node_constant(ECtx* c, int in)
{
    size_t const w = S(in)->w, n = S(in)->n;
    for (size_t i = 1; i < n; i++)
        if (memcmp(S(in)->data + i * w, S(in)->data, w) != 0) {
            c->err = OZO_ERR_GENERIC;
            break;
        }
    ENode* nd = new_node(c, S(in)->type == OZO_TYPE_SERIAL ? TR_CONSTANT_SERIAL : TR_CONSTANT_FIXED, in, 1);
    nd->hsz = ozo_varint_enc(nd->hdr, S(in)->n);
    int o = new_stream(c, S(in)->type, S(in)->w, 1, S(in)->data);
    nd->nbOut = 1;
    return o;
}

/* EI_flatpack (encode_flatpack_binding.c, encode_flatpack_kernel.c) */
static int node_flatpack(ECtx* c, int in)
{
    size_t const n = S(in)->n;
    uint8_t map[256] = { 0 }, alpha[256];
    for (size_t i = 0; i < n; i++) map[S(in)->data[i]] = 1;
    size_t na = 0;
    for (int s = 0; s < 256; s++)
        if (map[s]) { map[s] = (uint8_t)na; alpha[na++] = (uint8_t)s; }
    unsigned const nbBits = na <= 1 ? (unsigned)na : 1u + (unsigned)ozo_highbit32((uint32_t)na - 1);
    size_t const packed = n ? 1 + (nbBits * n) / 8 : 0;
    ENode* nd = new_node(c, TR_FLATPACK, in, 2);
    int a = new_stream(c, OZO_TYPE_SERIAL, 1, na, alpha);
    int p = new_stream(c, OZO_TYPE_SERIAL, 1, packed, NULL);
    nd->nbOut = 2;
    if (n) {
        /* LSB-first indices, then the marker bit: 1 + nbBits * n / 8 bytes */
        uint8_t* d = S(p)->data;
        memset(d + packed, 0, 8);
        BW b = { d, packed + 8, 0, 0, 0 };
        const uint8_t* const src = S(in)->data;
        for (size_t i = 0; i < n; i++) bw_add(&b, map[src[i]], nbBits);
        bw_close(&b);
    }
    return a;
}

/* Largest FSE table log the encoder may pick: the reference's
 * FSE_DEFAULT_TABLELOG (11, encode_entropy_binding.c:92-93). Tests raise it to
 * 12, the decoder's limit (FSE_MAX_TABLELOG, fse.h:732), to make frames that
 * exercise the widest fields; such frames are valid for the reference's
 * decoder but its encoder never writes them. */
static unsigned g_fseMaxTableLog = 11;

void ozo_test_set_fse_max_tablelog(unsigned tl) { g_fseMaxTableLog = tl == 12 ? 12u : 11u; }

/* Test hook, like the FSE one: Huffman tables may reach table log 12 (the
 * decoders' limit, HUF_TABLELOG_MAX) where the reference's encoder uses 11
 * (HUF_TABLELOG_DEFAULT). */
static unsigned g_hufMaxTableLog = 11;
void ozo_test_set_huf_max_tablelog(unsigned tl) { g_hufMaxTableLog = tl == 12 ? 12u : 11u; }

/* EI_fse_v2 (encode_entropy_binding.c:51-139): outputs normalized counts
 * (numeric i16) and the bitstream. */
static int node_fse(ECtx* c, int in, const Stats* st)
{
    size_t const n = S(in)->n;
    unsigned const nbStates = n < 1000 ? 2 : 4;
    ENode* nd = new_node(c, TR_FSE_V2, in, 2);
    nd->hdr[0] = (uint8_t)nbStates;
    size_t const nbBytes = (size_t)(ozo_nextpow2(n + 1) + 7) / 8;
    for (size_t b = 0; b < nbBytes; b++) nd->hdr[1 + b] = (uint8_t)(n >> (8 * b));
    nd->hsz = nbBytes + 1;
    unsigned const maxSV = st->maxSym;
    unsigned const tl = fse_optimal_tablelog(g_fseMaxTableLog, n, maxSV, 2);
    int16_t norm[256];
    if (fse_normalize(norm, tl, st->count, n, maxSV, 1)) c->err = OZO_ERR_GENERIC;
    int ns = new_stream(c, OZO_TYPE_NUMERIC, 2, maxSV + 1, NULL);
    for (unsigned s = 0; s <= maxSV; s++) ozo_wr16(S(ns)->data + 2 * s, (uint16_t)norm[s]);
    FseC* ct = (FseC*)malloc(sizeof(FseC));
    fse_build_ctable(ct, norm, maxSV, tl);
    size_t const cap = n + (n >> 7) + 512;
    uint8_t* tmp = (uint8_t*)malloc(cap);
    size_t const sz = fse_compress(tmp, cap, S(in)->data, n, ct, nbStates);
    if (sz == 0) c->err = OZO_ERR_GENERIC;
    new_stream(c, OZO_TYPE_SERIAL, 1, sz, tmp);
    nd->nbOut = 2;
    free(tmp);
    free(ct);
    return ns;
}

static int node_fse_ncount(ECtx* c, int in)
{
    size_t const nb = S(in)->n;
    int16_t norm[256];
    uint64_t sum = 0;
    for (size_t i = 0; i < nb; i++) {
        norm[i] = (int16_t)ozo_rd16(S(in)->data + 2 * i);
        sum += norm[i] == -1 ? 1 : (uint64_t)norm[i];
    }
    unsigned const tl = (unsigned)ozo_highbit64(sum);
    uint8_t buf[600];
    size_t const sz = fse_write_ncount(buf, norm, (unsigned)nb - 1, tl);
    ENode* nd = new_node(c, TR_FSE_NCOUNT, in, 1);
    int o = new_stream(c, OZO_TYPE_SERIAL, 1, sz, buf);
    nd->nbOut = 1;
    return o;
}

/* EI_huffman_v2 (encode_entropy_binding.c:191-286): weights (numeric u8)
 * and the 1X/4X bitstream. */
static int node_huf(ECtx* c, int in, const Stats* st)
{
    size_t const n = S(in)->n;
    unsigned const maxSV = st->maxSym;
    ENode* nd = new_node(c, TR_HUFFMAN_V2, in, 2);
    int ws = new_stream(c, OZO_TYPE_NUMERIC, 1, maxSV + 1, NULL);
    unsigned tl = fse_optimal_tablelog(g_hufMaxTableLog, n, maxSV, 1);
    HufC ct;
    tl = huf_build_ctable(&ct, st->count, maxSV, tl);
    for (unsigned s = 0; s <= maxSV; s++)
        S(ws)->data[s] = (uint8_t)(ct.nbBits[s] == 0 ? 0 : tl + 1 - ct.nbBits[s]);
    int const x4 = n > 1000;
    size_t const nbBytes = (size_t)(ozo_nextpow2(n + 1) + 7) / 8;
    nd->hdr[0] = (uint8_t)(x4 ? 1 : 0);
    for (size_t b = 0; b < nbBytes; b++) nd->hdr[1 + b] = (uint8_t)(n >> (8 * b));
    nd->hsz = nbBytes + 1;
    size_t const cap = n + (n >> 8) + 1024;
    uint8_t* tmp = (uint8_t*)malloc(cap);
    size_t const sz = x4 ? huf_compress4x(tmp, cap, S(in)->data, n, &ct) : huf_compress1x(tmp, cap, S(in)->data, n, &ct);
    if (sz == 0) c->err = OZO_ERR_GENERIC;
    new_stream(c, OZO_TYPE_SERIAL, 1, sz, tmp);
    nd->nbOut = 2;
    free(tmp);
    return ws;
}

/* EI_huffman_struct_v2 (encode_entropy_binding.c:287-367): weights (numeric
 * u8) and the stream table of 1 (up to 1000 symbols) or 4 streams; the
 * four streams hold size/4 + 1 symbols each, the last the rest
 * (encode_huffman_kernel.c:490-508). */
static int node_huf16(ECtx* c, int in, const unsigned* count, unsigned maxSV)
{
    size_t const n = S(in)->n;
    uint16_t* code = (uint16_t*)calloc((size_t)maxSV + 1, 2);
    uint16_t* nbb = (uint16_t*)calloc((size_t)maxSV + 1, 2);
    int const tl = lhuf_build_ctable(code, nbb, count, maxSV);
    if (tl < 0) c->err = OZO_ERR_GENERIC;
    ENode* nd = new_node(c, TR_HUFFMAN_STRUCT_V2, in, 2);
    int ws = new_stream(c, OZO_TYPE_NUMERIC, 1, (size_t)maxSV + 1, NULL);
    for (unsigned v = 0; v <= maxSV; v++) S(ws)->data[v] = (uint8_t)(nbb[v] == 0 ? 0 : tl + 1 - nbb[v]);
    int const x4 = n > 1000;
    size_t const nbBytes = (size_t)(ozo_nextpow2(n + 1) + 7) / 8;
    nd->hdr[0] = (uint8_t)(x4 ? 1 : 0);
    for (size_t b = 0; b < nbBytes; b++) nd->hdr[1 + b] = (uint8_t)(n >> (8 * b));
    nd->hsz = nbBytes + 1;
    size_t const cap = 2 * n + 32;
    uint8_t* tmp = (uint8_t*)malloc(cap);
    const uint8_t* const src = S(in)->data;
    size_t sz = 0;
    if (x4) {
        size_t off = 0, const_chunk = n / 4 + 1;
        for (int k = 0; k < 4 && tl >= 0; k++) {
            size_t const len = const_chunk < n - off ? const_chunk : n - off;
            size_t const r = lhuf_stream(tmp + sz, cap - sz, src + 2 * off, len, code, nbb);
            if (r == 0) { c->err = OZO_ERR_GENERIC; break; }
            sz += r;
            off += len;
        }
    } else if (tl >= 0) {
        sz = lhuf_stream(tmp, cap, src, n, code, nbb);
        if (sz == 0) c->err = OZO_ERR_GENERIC;
    }
    new_stream(c, OZO_TYPE_SERIAL, 1, sz, tmp);
    nd->nbOut = 2;
    free(tmp);
    free(code);
    free(nbb);
    return ws;
}

/* tokenizeImpl (encode_tokenize_binding.c:127-215): alphabet in order of
 * first occurrence (ascending unsigned order when sorted), indices of 1, 2
 * or 4 bytes by alphabet size. */
static int cmp_u64(const void* a, const void* b)
{
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : x > y;
}
static int node_tokenize(ECtx* c, int in, int sorted)
{
    size_t const w = S(in)->w, n = S(in)->n;
    /* open-addressing map token -> first-occurrence index */
    size_t cap = 16;
    while (cap < 2 * n + 16) cap <<= 1;
    uint64_t* keys = (uint64_t*)malloc(cap * 8);
    uint32_t* vals = (uint32_t*)malloc(cap * 4);
    uint8_t* used = (uint8_t*)calloc(cap, 1);
    uint64_t* alpha = (uint64_t*)malloc((n + 1) * 8);
    uint32_t* idx = (uint32_t*)malloc((n + 1) * 4);
    size_t na = 0;
    for (size_t i = 0; i < n; i++) {
        uint64_t const t = rd(S(in)->data + i * w, w);
        size_t h = (size_t)((t * 0x9E3779B97F4A7C15ull) >> 20) & (cap - 1);
        while (used[h] && keys[h] != t) h = (h + 1) & (cap - 1);
        if (!used[h]) { used[h] = 1; keys[h] = t; vals[h] = (uint32_t)na; alpha[na++] = t; }
        idx[i] = vals[h];
    }
    if (sorted) {
        uint64_t* sortedA = (uint64_t*)malloc((na + 1) * 8);
        memcpy(sortedA, alpha, na * 8);
        qsort(sortedA, na, 8, cmp_u64);
        uint32_t* remap = (uint32_t*)malloc((na + 1) * 4);
        for (size_t k = 0; k < na; k++) {
            uint64_t t = sortedA[k];
            size_t h = (size_t)((t * 0x9E3779B97F4A7C15ull) >> 20) & (cap - 1);
            while (keys[h] != t) h = (h + 1) & (cap - 1);
            remap[vals[h]] = (uint32_t)k;
        }
        for (size_t i = 0; i < n; i++) idx[i] = remap[idx[i]];
        memcpy(alpha, sortedA, na * 8);
        free(sortedA);
        free(remap);
    }
    size_t const iw = na <= 256 ? 1 : (na <= 65536 ? 2 : 4);
    /* struct input: tokenize_struct, first-occurrence order only */
    ENode* nd = new_node(c, S(in)->type == OZO_TYPE_STRUCT ? TR_TOKENIZE_FIXED : TR_TOKENIZE_NUMERIC, in, 2);
    int a = new_stream(c, S(in)->type, w, na, NULL);
    for (size_t k = 0; k < na; k++) wr(S(a)->data + k * w, alpha[k], w);
    int o = new_stream(c, OZO_TYPE_NUMERIC, iw, n, NULL);
    for (size_t i = 0; i < n; i++) wr(S(o)->data + i * iw, idx[i], iw);
    nd->nbOut = 2;
    free(keys); free(vals); free(used); free(alpha); free(idx);
    return a;
}

/* EI_bfloat16_deconstruct (encode_float_deconstruct_binding.c:14-80):
 * header = element type; outputs sign|fraction (struct, width 1) and
 * exponent (serial). */
static int node_bf16(ECtx* c, int in)
{
    size_t const n = S(in)->n;
    ENode* nd = new_node(c, TR_FLOAT_DECONSTRUCT, in, 2);
    nd->hdr[0] = 1;
    nd->hsz = 1;
    int sf = new_stream(c, OZO_TYPE_STRUCT, 1, n, NULL);
    int ex = new_stream(c, OZO_TYPE_SERIAL, 1, n, NULL);
    for (size_t i = 0; i < n; i++) {
        uint16_t x = ozo_rd16(S(in)->data + 2 * i);
        S(sf)->data[i] = (uint8_t)(((x >> 15) & 1) | ((x & 0x7F) << 1));
        S(ex)->data[i] = (uint8_t)(x >> 7);
    }
    nd->nbOut = 2;
    return sf;
}

/* entropyCompressChunk for serial chunks (encode_entropy_binding.c:602-762).
 * mode: 0 FSE graph (EBM_fse), 1 Huffman graph (EBM_huf), 2 entropy graph
 * (EBM_any: FSE or Huffman by resolveMode, encode_entropy_binding.c:527-548). */
static int entropy_chunk(ECtx* c, int sid, int hufMode, SuccList* succ)
{
    size_t const n = S(sid)->n;
    if (n <= 1) { succ_add(succ, G_STORE, sid, NULL); return 0; }
    Stats st;
    stats_init(&st, S(sid)->data, n);
    if (st.card == 1) { succ_add(succ, G_CONSTANT, sid, NULL); return 0; }
    size_t entropySize;
    if (hufMode == 1) {
        entropySize = stats_huf_fast(&st);
    } else {
        volatile double e = stats_entropy(&st);
        volatile double prod = e * (double)n;
        volatile double sum = prod + 7;
        entropySize = (size_t)sum / 8;
    }
    size_t const header = st.card / 4 > 10 ? st.card / 4 : 10;
    size_t baseline = entropySize + header;
    if (n < baseline) baseline = n;
    size_t const flat = stats_flatpacked(&st), bp = stats_bitpacked(&st);
    if (flat < bp) {
        if (flat < baseline) { succ_add(succ, G_FLATPACK, sid, NULL); return 0; }
    } else if (bp < baseline) {
        succ_add(succ, G_BITPACK, sid, NULL);
        return 0;
    }
    if (n <= baseline) { succ_add(succ, G_STORE, sid, NULL); return 0; }
    if (hufMode == 2) {
        /* the FSE size is the entropy estimate above */
        hufMode = entropySize + n / 32 < stats_huf_fast(&st) ? 0 : 1;
    }
    if (hufMode) {
        int w = node_huf(c, sid, &st);
        succ_add(succ, G_FSE, w, NULL);
        succ_add(succ, G_STORE, w + 1, NULL);
    } else {
        int ns = node_fse(c, sid, &st);
        succ_add(succ, G_FSE_NCOUNT, ns, NULL);
        succ_add(succ, G_STORE, ns + 1, NULL);
    }
    return 0;
}

/* entropyCompressChunk for 16-bit struct chunks (encode_entropy_binding.c:
 * 612-681): constant, bitpack, store, tokenize (fewer than 256 distinct
 * values) or huffman_struct_v2, whatever the graph's backend mode. */
static int entropy_chunk16(ECtx* c, int sid, SuccList* succ)
{
    size_t const n = S(sid)->n;
    if (n <= 1) { succ_add(succ, G_STORE, sid, NULL); return 0; }
    unsigned* count = (unsigned*)calloc(65536, sizeof(unsigned));
    unsigned maxSym = 0;
    for (size_t i = 0; i < n; i++) {
        unsigned const v = ozo_rd16(S(sid)->data + 2 * i);
        count[v]++;
        if (v > maxSym) maxSym = v;
    }
    if (count[maxSym] == n) { free(count); succ_add(succ, G_CONSTANT, sid, NULL); return 0; }
    size_t card = 0;
    for (unsigned v = 0; v <= maxSym; v++) card += count[v] > 0;
    double entropy = calc_entropy(count, maxSym, n);
    if (1 > entropy) entropy = 1;
    volatile double prod = entropy * (double)n;
    volatile double sum = prod + 7;
    size_t const entropySize = (size_t)sum / 8;
    size_t const header = maxSym / 4 > 100 ? maxSym / 4 : 100;
    size_t const huffSize = entropySize + header, storeSize = 2 * n;
    size_t const nbBits = (size_t)ozo_nextpow2((uint64_t)maxSym + 1);
    size_t const bitpackSize = (n * nbBits + 7) / 8 + 2;
    if (bitpackSize <= huffSize && bitpackSize < storeSize) {
        /* runBitpack: interpret the tokens as little-endian numbers */
        succ_add(succ, G_BITPACK, node_conv_struct_to_num(c, sid), NULL);
    } else if (entropy > 15 || huffSize >= storeSize) {
        succ_add(succ, G_STORE, sid, NULL);
    } else if (card < 256) {
        int const a = node_tokenize(c, sid, 0);
        if (nbBits < 16) succ_add(succ, G_BITPACK, node_conv_struct_to_num(c, a), NULL);
        else succ_add(succ, G_STORE, a, NULL);
        succ_add(succ, G_HUF, a + 1, NULL);
    } else {
        int const w = node_huf16(c, sid, count, maxSym);
        succ_add(succ, G_FSE, w, NULL);
        succ_add(succ, G_STORE, w + 1, NULL);
    }
    free(count);
    return 0;
}

/* entropyDynamicGraph (encode_entropy_binding.c:765-868) for FSE / Huffman
 * / entropy */
static int graph_entropy(ECtx* c, int sid, int hufMode)
{
    SuccList succ = { 0 };
    /* doEntropyConversion (encode_entropy_binding.c:764-810): eltWidth 1
     * goes to serial, numeric eltWidth 2 to struct; other widths are
     * rejected */
    if (S(sid)->w == 1 && S(sid)->type != OZO_TYPE_SERIAL)
        sid = S(sid)->type == OZO_TYPE_NUMERIC ? node_conv_num_to_serial(c, sid) : node_conv_struct_to_serial(c, sid);
    else if (S(sid)->w == 2 && S(sid)->type == OZO_TYPE_NUMERIC)
        sid = node_conv_num_to_struct(c, sid);
    if (S(sid)->w != 1 && S(sid)->w != 2) { c->err = OZO_ERR_UNSUPPORTED; return -1; }
    int const wide = S(sid)->w == 2;
    size_t const n = S(sid)->n;
    size_t const kChunk = 1 << 15;
    if (n < 100000) {
        if (wide) entropy_chunk16(c, sid, &succ);
        else entropy_chunk(c, sid, hufMode, &succ);
    } else {
        size_t const nb = (n + kChunk - 1) / kChunk;
        size_t* sizes = (size_t*)malloc(nb * sizeof(size_t));
        for (size_t i = 0; i + 1 < nb; i++) sizes[i] = kChunk;
        sizes[nb - 1] = n - (nb - 1) * kChunk;
        int first = node_splitn(c, sid, sizes, nb);
        free(sizes);
        for (size_t i = 0; i < nb; i++) {
            if (wide) entropy_chunk16(c, first + (int)i, &succ);
            else entropy_chunk(c, first + (int)i, hufMode, &succ);
        }
    }
    return run_succs(c, &succ);
}

static int run_graph(ECtx* c, int g, int sid, const void* arg)
{
    SuccList succ = { 0 };
    switch (g) {
        case G_SERIAL_STORE:
            sid = convert_for(c, sid, OZO_TYPE_SERIAL);
            S(sid)->store = 1;
            return 0;
        case G_STORE:
            /* public store: forwards to the type-dispatching store */
            return run_successor(c, G_SERIAL_STORE, sid, NULL);
        case G_FSE:
            sid = convert_for(c, sid, OZO_TYPE_SERIAL);
            return graph_entropy(c, sid, 0);
        case G_HUF:
            return graph_entropy(c, sid, 1);
        case G_ENTROPY:
            return graph_entropy(c, sid, 2);
        case G_CONSTANT: {
            /* the constant graph takes serial or struct input: numbers are
             * converted to struct first (graph_registry.c:132) */
            sid = convert_for(c, sid, OZO_TYPE_SERIAL | OZO_TYPE_STRUCT);
            int o = node_constant(c, sid);
            return run_successor(c, G_SERIAL_STORE, o, NULL);
        }
        case G_BITPACK: {
            int o = node_bitpack(c, sid, S(sid)->type == OZO_TYPE_NUMERIC ? TR_BITPACK_INT : TR_BITPACK_SERIAL);
            return run_successor(c, G_SERIAL_STORE, o, NULL);
        }
        case G_FLATPACK: {
            sid = convert_for(c, sid, OZO_TYPE_SERIAL);
            int a = node_flatpack(c, sid);
            succ_add(&succ, G_SERIAL_STORE, a, NULL);
            succ_add(&succ, G_SERIAL_STORE, a + 1, NULL);
            return run_succs(c, &succ);
        }
        case G_FSE_NCOUNT: {
            int o = node_fse_ncount(c, sid);
            return run_successor(c, G_SERIAL_STORE, o, NULL);
        }
        case G_TSPLIT_FSE:
        case G_TSPLIT_STORE: {
            sid = convert_for(c, sid, OZO_TYPE_STRUCT);
            size_t const W = S(sid)->w;
            int first = node_tsplit(c, sid);
            for (size_t b = 0; b < W; b++) succ_add(&succ, g == G_TSPLIT_FSE ? G_FSE : G_STORE, first + (int)b, NULL);
            return run_succs(c, &succ);
        }
        case G_BITPACK_HUF: {
            sid = convert_for(c, sid, OZO_TYPE_NUMERIC);
            int o = node_bitpack(c, sid, TR_BITPACK_INT);
            return run_successor(c, G_HUF, o, NULL);
        }
        case G_TOKENIZE:
        case G_TOKENIZE_SORTED: {
            sid = convert_for(c, sid, OZO_TYPE_NUMERIC);
            int a = node_tokenize(c, sid, g == G_TOKENIZE_SORTED);
            succ_add(&succ, G_STORE, a, NULL);
            succ_add(&succ, G_BITPACK_HUF, a + 1, NULL);
            return run_succs(c, &succ);
        }
        case G_BF16: {
            sid = convert_for(c, sid, OZO_TYPE_NUMERIC);
            int sf = node_bf16(c, sid);
            succ_add(&succ, G_STORE, sf, NULL);
            succ_add(&succ, G_FSE, sf + 1, NULL);
            return run_succs(c, &succ);
        }
        case G_CHAIN: {
            /* pipeline: arg = zero-terminated list of steps, then a final graph */
            const int* steps = (const int*)arg;
            int cur = sid;
            for (; *steps > 0 && *steps < 100; steps++) {
                if (steps != (const int*)arg) {
                    /* each pipeline hop is a successor: small streams are stored */
                    if (S(cur)->n * S(cur)->w < 10) return run_successor(c, G_STORE, cur, NULL);
                }
                switch (*steps) {
                    case 1: cur = node_delta(c, convert_for(c, cur, OZO_TYPE_NUMERIC)); break;
                    case 2: cur = node_zigzag(c, convert_for(c, cur, OZO_TYPE_NUMERIC)); break;
                    case 3: cur = node_conv_num_to_struct(c, convert_for(c, cur, OZO_TYPE_NUMERIC)); break;
                    default: c->err = OZO_ERR_UNSUPPORTED; return -1;
                }
            }
            return run_successor(c, *steps - 100, cur, NULL);
        }
        default:
            c->err = OZO_ERR_UNSUPPORTED;
            return -1;
    }
}

/* CCTX_runSuccessor_internal (cctx.c:1116-1183): small single inputs are
 * stored; everything else runs its graph. */
static int run_successor(ECtx* c, int g, int sid, const void* arg)
{
    if (c->err) return -1;
    if (g != G_SERIAL_STORE && S(sid)->n * S(sid)->w < 10) g = G_STORE;
    if (g == G_STORE && S(sid)->n * S(sid)->w < 10) return run_graph(c, G_SERIAL_STORE, sid, NULL);
    return run_graph(c, g, sid, arg);
}

/* ------------------------------------------------------------------ */
/* frame writer (src/openzl/compress/encode_frameheader.c:441-834) */
typedef struct {
    uint8_t* p;
    size_t pos, cap;
    int overflow;
} Out;

static void out_push(Out* o, uint8_t b)
{
    if (o->pos < o->cap) o->p[o->pos] = b;
    else o->overflow = 1;
    o->pos++;
}
static void out_bytes(Out* o, const uint8_t* src, size_t n)
{
    if (n && o->pos + n <= o->cap) memcpy(o->p + o->pos, src, n);
    else if (n) o->overflow = 1;
    o->pos += n;
}
static void out_varint(Out* o, uint64_t v)
{
    uint8_t t[10];
    size_t n = ozo_varint_enc(t, v);
    for (size_t i = 0; i < n; i++) out_push(o, t[i]);
}
static void out_bits(Out* o, const uint32_t* v, size_t n, int nbBits)
{
    size_t const bytes = (n * (size_t)nbBits + 7) / 8;
    size_t const base = o->pos;
    for (size_t i = 0; i < bytes; i++) out_push(o, 0);
    if (o->overflow) return;
    for (size_t i = 0; i < n; i++) {
        size_t bit = i * (size_t)nbBits;
        for (int b = 0; b < nbBits; b++, bit++)
            if ((v[i] >> b) & 1) o->p[base + (bit >> 3)] |= (uint8_t)(1u << (bit & 7));
    }
}

static int64_t write_frame(ECtx* c, uint8_t* dst, size_t cap, int checksums)
{
    Out o = { dst, 0, cap, 0 };
    EStream* in0 = S(0);
    /* frame header */
    uint32_t const magic = OZO_MAGIC_BASE + 23;
    for (int b = 0; b < 4; b++) out_push(&o, (uint8_t)(magic >> (8 * b)));
    out_push(&o, (uint8_t)(checksums ? 3 : 0));
    static const uint8_t typeCode[9] = { 0, 0, 1, 0, 2, 0, 0, 0, 3 };
    out_push(&o, (uint8_t)(1 | (typeCode[in0->type] << 4)));
    out_varint(&o, in0->n * in0->w + 1);
    if (checksums) {
        if (o.overflow) return -OZO_ERR_DST_SIZE;
        out_push(&o, (uint8_t)(ozo_xxh3_64(dst, o.pos) & 255));
    }
    size_t const blockStart = o.pos;
    /* chunk header: decoders in reverse creation order */
    size_t const nd = c->nn;
    size_t nbStored = 0;
    for (size_t i = 0; i < c->ns; i++) nbStored += c->s[i].store;
    out_varint(&o, nd + 1);
    out_varint(&o, nbStored);
    uint32_t* a = (uint32_t*)calloc(nd + c->ns + 1, 4);
    for (size_t u = 0; u < nd; u++) a[u] = 0;
    out_bits(&o, a, nd, 1);
    for (size_t u = 0; u < nd; u++) a[u] = c->nd[nd - 1 - u].trid;
    out_bits(&o, a, nd, ozo_nextpow2(TR_END));
    for (size_t u = 0; u < nd; u++) a[u] = c->nd[nd - 1 - u].hsz > 0;
    out_bits(&o, a, nd, 1);
    for (size_t u = 0; u < nd; u++)
        if (c->nd[nd - 1 - u].hsz) out_varint(&o, c->nd[nd - 1 - u].hsz - 1);
    for (size_t u = 0; u < nd; u++) {
        ENode* x = &c->nd[nd - 1 - u];
        a[u] = (x->nbOut - x->nbSO) > 0;
    }
    out_bits(&o, a, nd, 1);
    for (size_t u = 0; u < nd; u++) {
        ENode* x = &c->nd[nd - 1 - u];
        if (x->nbOut - x->nbSO > 0) out_varint(&o, (uint64_t)(x->nbOut - x->nbSO - 1));
    }
    for (size_t u = 0; u < nd; u++) a[u] = 0; /* single-input codecs only */
    out_bits(&o, a, nd, 1);
    for (size_t u = 0; u < nd; u++) {
        ENode* x = &c->nd[nd - 1 - u];
        a[u] = (uint32_t)(x->outStart - x->in) - 1;
    }
    out_bits(&o, a, nd, ozo_nextpow2(nd + nbStored));
    for (size_t i = c->ns; i-- > 0;)
        if (c->s[i].store) out_varint(&o, c->s[i].n * c->s[i].w);
    free(a);
    /* codec headers, then stored streams */
    for (size_t u = 0; u < nd; u++) {
        ENode* x = &c->nd[nd - 1 - u];
        for (size_t b = 0; b < x->hsz; b++) out_push(&o, x->hdr[b]);
    }
    for (size_t i = c->ns; i-- > 0;)
        if (c->s[i].store)
            out_bytes(&o, c->s[i].data, c->s[i].n * c->s[i].w);
    if (checksums) {
        uint32_t const h = (uint32_t)ozo_xxh3_64(in0->data, in0->n * in0->w);
        for (int b = 0; b < 4; b++) out_push(&o, (uint8_t)(h >> (8 * b)));
        if (o.overflow) return -OZO_ERR_DST_SIZE;
        uint32_t const hc = (uint32_t)ozo_xxh3_64(dst + blockStart, o.pos - blockStart);
        for (int b = 0; b < 4; b++) out_push(&o, (uint8_t)(hc >> (8 * b)));
    }
    out_push(&o, 0);
    if (o.overflow) return -OZO_ERR_DST_SIZE;
    return (int64_t)o.pos;
}

size_t ozo_compress_bound(size_t srcSize) { return srcSize * 2 + 65536; }

int64_t ozo_compress(int recipe, const void* src, size_t nbElts, int eltWidth, void* dst, size_t dstCap,
                     int checksums)
{
    ECtx c;
    memset(&c, 0, sizeof(c));
    int const type = eltWidth ? OZO_TYPE_NUMERIC : OZO_TYPE_SERIAL;
    size_t const w = eltWidth ? (size_t)eltWidth : 1;
    int in = new_stream(&c, type, w, nbElts, (const uint8_t*)src);
    static const int chainDZ_TS[] = { 1, 2, 3, 100 + G_TSPLIT_FSE };
    static const int chainDZ_BH[] = { 1, 2, 100 + G_BITPACK_HUF };
    static const int chainD_TS[] = { 1, 3, 100 + G_TSPLIT_FSE };
    static const int chainD_BH[] = { 1, 100 + G_BITPACK_HUF };
    static const int chainD_ST[] = { 1, 100 + G_STORE };
    static const int chainZ_ST[] = { 2, 100 + G_STORE };
    static const int chainB_ST[] = { 100 + G_BITPACK };
    static const int chainT_ST[] = { 3, 100 + G_TSPLIT_STORE };
    int rc;
    switch (recipe) {
        case R_STORE: rc = run_successor(&c, G_STORE, in, NULL); break;
        case R_DZ_TSPLIT_FSE: rc = run_successor(&c, G_CHAIN, in, chainDZ_TS); break;
        case R_DZ_BITPACK_HUF: rc = run_successor(&c, G_CHAIN, in, chainDZ_BH); break;
        case R_D_TSPLIT_FSE: rc = run_successor(&c, G_CHAIN, in, chainD_TS); break;
        case R_D_BITPACK_HUF: rc = run_successor(&c, G_CHAIN, in, chainD_BH); break;
        case R_FSE: rc = run_successor(&c, G_FSE, in, NULL); break;
        case R_TOKENIZE: rc = run_successor(&c, G_TOKENIZE, in, NULL); break;
        case R_TOKENIZE_SORTED: rc = run_successor(&c, G_TOKENIZE_SORTED, in, NULL); break;
        case R_BF16: rc = run_successor(&c, G_BF16, in, NULL); break;
        case R_HUFFMAN: rc = run_successor(&c, G_HUF, in, NULL); break;
        case R_ENTROPY: rc = run_successor(&c, G_ENTROPY, in, NULL); break;
        case R_DELTA_STORE: rc = run_successor(&c, G_CHAIN, in, chainD_ST); break;
        case R_ZIGZAG_STORE: rc = run_successor(&c, G_CHAIN, in, chainZ_ST); break;
        case R_BITPACK_STORE: rc = run_successor(&c, G_CHAIN, in, chainB_ST); break;
        case R_TSPLIT_STORE: rc = run_successor(&c, G_CHAIN, in, chainT_ST); break;
        case R_CONSTANT: rc = run_successor(&c, G_CONSTANT, in, NULL); break;
        case R_FLATPACK: rc = run_successor(&c, G_FLATPACK, in, NULL); break;
        case R_BITPACK_GRAPH: rc = run_successor(&c, G_BITPACK, in, NULL); break;
        default: rc = -1; c.err = OZO_ERR_UNSUPPORTED;
    }
    int64_t ret;
    if (rc || c.err) ret = -(int64_t)(c.err ? c.err : OZO_ERR_GENERIC);
    else ret = write_frame(&c, (uint8_t*)dst, dstCap, checksums);
    for (size_t i = 0; i < c.ns; i++) free(c.s[i].data);
    free(c.s);
    free(c.nd);
    return ret;
}

/* Test entry point: the tokenize node alone (encoder known answers):
 * alphabet (na values of width w) and indices (n of width *iw). */
int64_t ozo_tokenize(const void* src, size_t n, int w, int sorted, void* alphaOut, void* idxOut, int* iwOut)
{
    ECtx ctx;
    ECtx* const c = &ctx;
    memset(c, 0, sizeof(*c));
    int in = new_stream(c, OZO_TYPE_NUMERIC, (size_t)w, n, (const uint8_t*)src);
    int a = node_tokenize(c, in, sorted);
    size_t const na = S(a)->n;
    memcpy(alphaOut, S(a)->data, na * (size_t)w);
    memcpy(idxOut, S(a + 1)->data, n * S(a + 1)->w);
    *iwOut = (int)S(a + 1)->w;
    for (size_t i = 0; i < c->ns; i++) free(c->s[i].data);
    free(c->s);
    free(c->nd);
    return (int64_t)na;
}

