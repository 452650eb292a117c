/* CPU restatement of OpenZL's universal decoder for the numeric codec graph
 * (formats 21-23). Test infrastructure only: the checker the GPU decoder is
 * compared against. Each function cites the reference code it restates. */
#include <stdio.h>

#include <string.h>

#include "ozo_internal.h"

typedef struct {
    int type;          /* OZO_TYPE_* */
    size_t w;          /* element width in bytes */
    size_t n;          /* number of elements (string streams: content bytes) */
    const uint8_t* p;  /* content */
    uint8_t* own;      /* owned allocation, if any */
    int filled;
    uint32_t* lens;    /* string streams: the length of each string (owned) */
    size_t nbStrings;
} OStream;

static void ost_free(OStream* s)
{
    free(s->own);
    free(s->lens);
    memset(s, 0, sizeof(*s));
}
static uint8_t* ost_alloc(OStream* s, int type, size_t w, size_t n)
{
    s->type = type;
    s->w = w;
    s->n = n;
    s->own = (uint8_t*)malloc(n * w + 16);
    s->p = s->own;
    s->filled = 1;
    return s->own;
}
static void ost_ref(OStream* s, int type, size_t w, size_t n, const uint8_t* p)
{
    s->type = type;
    s->w = w;
    s->n = n;
    s->p = p;
    s->own = NULL;
    s->filled = 1;
}

/* ---------------------------------------------------------------------
 * LSB-first bitpack decode (src/openzl/codecs/bitpack/spec.md,
 * common_bitpack_kernel.c). Element i occupies bits [i*nbBits, (i+1)*nbBits)
 * of the little-endian byte stream. Returns bytes consumed.
 * ------------------------------------------------------------------- */
static uint64_t le64_at(const uint8_t* p)
{
    uint64_t v;
    memcpy(&v, p, 8);
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_BIG_ENDIAN__
    v = __builtin_bswap64(v);
#endif
    return v;
}

static size_t bitunpack(uint64_t* dst, size_t n, const uint8_t* src, size_t srcSize, int nbBits)
{
    size_t const need = (n * (size_t)nbBits + 7) / 8;
    if (need > srcSize) return (size_t)-1;
    uint64_t const mask = nbBits >= 64 ? ~0ull : ((1ull << nbBits) - 1);
    for (size_t i = 0; i < n; i++) {
        size_t const bit = i * (size_t)nbBits;
        size_t const b = bit >> 3;
        unsigned const sh = (unsigned)(bit & 7);
        if (sh + (unsigned)nbBits <= 64 && b + 8 <= srcSize) {
            dst[i] = (le64_at(src + b) >> sh) & mask;
            continue;
        }
        uint64_t v = 0;
        for (int k = 0; k < nbBits; k++) {
            size_t q = bit + (size_t)k;
            v |= (uint64_t)((src[q >> 3] >> (q & 7)) & 1) << k;
        }
        dst[i] = v;
    }
    return need;
}

/* ---------------------------------------------------------------------
 * Backward bit reader shared by FSE and Huffman (src/openzl/fse/bitstream.h):
 * the stream is read from its last byte towards its first; the highest set
 * bit of the last byte is an end marker; fields are read most significant
 * bit first. Bits below position 0 read as zero.
 * ------------------------------------------------------------------- */
/* The reader keeps 64 bits of the stream starting at bit index `base` in
 * `cont`; fields below position 0 read as zero. */
typedef struct {
    const uint8_t* src;
    size_t size;
    int64_t pos;
    int64_t base;
    uint64_t cont;
} BCont;

static inline void bc_fill(BCont* r)
{
    int64_t b = ((r->pos + 7) >> 3) - 8;
    if (b < 0) b = 0;
    r->base = b * 8;
    if ((size_t)b + 8 <= r->size) {
        r->cont = le64_at(r->src + b);
    } else {
        uint64_t v = 0;
        for (size_t k = 0; (size_t)b + k < r->size && k < 8; k++) v |= (uint64_t)r->src[b + k] << (8 * k);
        r->cont = v;
    }
}
static inline int bc_init(BCont* r, const uint8_t* src, size_t size)
{
    if (size == 0 || src[size - 1] == 0) return -1;
    r->src = src;
    r->size = size;
    r->pos = (int64_t)(size - 1) * 8 + ozo_highbit32(src[size - 1]);
    bc_fill(r);
    return 0;
}
static inline uint32_t bc_peek(const BCont* r, int nb)
{
    int64_t const sh = r->pos - nb - r->base;
    uint64_t const v = sh >= 0 ? (r->cont >> sh) : (r->cont << -sh);
    return (uint32_t)(v & ((1ull << nb) - 1));
}
static inline void bc_skip(BCont* r, int nb)
{
    r->pos -= nb;
    if (r->pos - r->base < 32 && r->base > 0) bc_fill(r);
}

/* Fast reader for the bulk of a stream (the same bits as BCont): `c` holds
 * the 8 stream bytes at `p`, of which the top `used` bits have been read. A
 * refill moves p down by the whole bytes read. The fast loops run only while
 * p is at least 8 bytes above the stream's first byte, so a group of up to
 * 56 bits and its refill never reach position 0; the rest of the stream
 * continues on BCont (bc_at). */
typedef struct {
    const uint8_t* p;
    uint64_t c;
    unsigned used;
} BFast;

static inline void bf_from(BFast* f, const uint8_t* src, int64_t pos) /* pos >= 64 */
{
    int64_t const top = (pos + 7) >> 3; /* bytes [0, top) hold the unread bits */
    f->p = src + top - 8;
    f->c = le64_at(f->p);
    f->used = (unsigned)(top * 8 - pos);
}
static inline int64_t bf_pos(const BFast* f, const uint8_t* src)
{
    return (int64_t)(f->p - src) * 8 + 64 - (int64_t)f->used;
}
/* nb in [0, 32]: the next nb bits (0 for nb = 0) */
static inline uint32_t bf_read(BFast* f, unsigned nb)
{
    uint32_t const v = (uint32_t)(((f->c << f->used) >> 1) >> (63 - nb));
    f->used += nb;
    return v;
}
static inline uint32_t bf_peek(const BFast* f, unsigned nb) { return (uint32_t)((f->c << f->used) >> (64 - nb)); }
static inline void bf_refill(BFast* f)
{
    f->p -= f->used >> 3;
    f->used &= 7;
    f->c = le64_at(f->p);
}
static inline void bc_at(BCont* r, const uint8_t* src, size_t size, int64_t pos)
{
    r->src = src;
    r->size = size;
    r->pos = pos;
    bc_fill(r);
}

/* ---------------------------------------------------------------------
 * FSE normalized-count header (src/openzl/fse/common/entropy_common.c:42-185,
 * FSE_readNCount): 4 bits tableLog-5, then per symbol a variable-width count
 * with a 2-bit repeat code for runs of zero counts. Returns bytes read.
 * ------------------------------------------------------------------- */
static int64_t fse_read_ncount(int16_t* norm, unsigned* maxSV, unsigned* tableLog,
                               const uint8_t* src, size_t size)
{
    size_t bitpos = 0;
    size_t const total = size * 8;
#define GETBITS(nb) ({ uint32_t _v = 0; for (int _i = 0; _i < (nb); _i++) { size_t _q = bitpos + _i; \
        _v |= (uint32_t)(_q < total ? ((src[_q >> 3] >> (_q & 7)) & 1) : 0) << _i; } _v; })
    unsigned const maxSV1 = *maxSV + 1;
    memset(norm, 0, maxSV1 * sizeof(int16_t));
    if (size < 1) return -OZO_ERR_CORRUPTION;
    int nbBits = (int)GETBITS(4) + 5;
    bitpos += 4;
    if (nbBits > 15) return -OZO_ERR_CORRUPTION;
    *tableLog = (unsigned)nbBits;
    int remaining = (1 << nbBits) + 1;
    int threshold = 1 << nbBits;
    nbBits++;
    unsigned charnum = 0;
    int previous0 = 0;
    while (remaining > 1 && charnum < maxSV1) {
        if (previous0) {
            unsigned n0 = charnum;
            while (GETBITS(2) == 3) { n0 += 3; bitpos += 2; }
            n0 += GETBITS(2);
            bitpos += 2;
            if (n0 > maxSV1) return -OZO_ERR_CORRUPTION;
            charnum = n0;
            if (charnum >= maxSV1) break;
        }
        int const max = (2 * threshold - 1) - remaining;
        int count;
        uint32_t const low = GETBITS(nbBits - 1);
        if ((int)low < max) {
            count = (int)low;
            bitpos += (size_t)(nbBits - 1);
        } else {
            count = (int)GETBITS(nbBits);
            if (count >= threshold) count -= max;
            bitpos += (size_t)nbBits;
        }
        count--;
        remaining -= count < 0 ? -count : count;
        norm[charnum++] = (int16_t)count;
        previous0 = !count;
        while (remaining < threshold) {
            nbBits--;
            threshold >>= 1;
        }
    }
#undef GETBITS
    if (remaining != 1) return -OZO_ERR_CORRUPTION;
    if (charnum > maxSV1) return -OZO_ERR_CORRUPTION;
    if (bitpos > total) return -OZO_ERR_CORRUPTION;
    *maxSV = charnum - 1;
    return (int64_t)((bitpos + 7) >> 3);
}

/* FSE decoding table (src/openzl/fse/decompress/fse_decompress.c:73-171). */
typedef struct {
    uint16_t newState;
    uint8_t symbol;
    uint8_t nbBits;
} FseD;

static int fse_build_dtable(FseD* dt, const int16_t* norm, unsigned maxSV, unsigned tableLog)
{
    uint32_t const tableSize = 1u << tableLog;
    uint32_t const mask = tableSize - 1;
    uint32_t const step = (tableSize >> 1) + (tableSize >> 3) + 3;
    uint32_t high = tableSize - 1;
    uint16_t next[256];
    for (unsigned s = 0; s <= maxSV; s++) {
        if (norm[s] == -1) {
            dt[high--].symbol = (uint8_t)s;
            next[s] = 1;
        } else {
            next[s] = (uint16_t)norm[s];
        }
    }
    uint32_t pos = 0;
    for (unsigned s = 0; s <= maxSV; s++) {
        for (int i = 0; i < norm[s]; i++) {
            dt[pos].symbol = (uint8_t)s;
            do { pos = (pos + step) & mask; } while (pos > high);
        }
    }
    if (pos != 0) return -1;
    for (uint32_t u = 0; u < tableSize; u++) {
        uint8_t const s = dt[u].symbol;
        uint32_t const x = next[s]++;
        dt[u].nbBits = (uint8_t)(tableLog - (unsigned)ozo_highbit32(x));
        dt[u].newState = (uint16_t)((x << dt[u].nbBits) - tableSize);
    }
    return 0;
}

/* Interleaved-state FSE decode (src/openzl/fse/decompress/fse_decompress.c:
 * 255-337): nbStates states read their initial values in order, symbol i is
 * produced by state i % nbStates, and every symbol except the last one of
 * each state is followed by that state's transition. */
static int fse_decode(uint8_t* dst, size_t dstSize, const uint8_t* src, size_t srcSize,
                      const FseD* dt, unsigned tableLog, unsigned nbStates)
{
    BCont r;
    if (bc_init(&r, src, srcSize)) return -OZO_ERR_CORRUPTION;
    uint32_t st[4];
    for (unsigned k = 0; k < nbStates; k++) {
        st[k] = bc_peek(&r, (int)tableLog);
        bc_skip(&r, (int)tableLog);
    }
    if (dstSize < nbStates) return -OZO_ERR_CORRUPTION;
    size_t const lastTransition = dstSize - nbStates;
    size_t i = 0;
    /* bulk: four symbols (at most 48 bits, tableLog <= 12) per refill */
    if (r.pos >= 64 && tableLog <= 12) {
        BFast f;
        bf_from(&f, src, r.pos);
        if (nbStates == 4) {
            uint32_t s0 = st[0], s1 = st[1], s2 = st[2], s3 = st[3];
            while (i + 4 <= lastTransition && f.p - src >= 8) {
                FseD const e0 = dt[s0], e1 = dt[s1], e2 = dt[s2], e3 = dt[s3];
                dst[i] = e0.symbol;
                dst[i + 1] = e1.symbol;
                dst[i + 2] = e2.symbol;
                dst[i + 3] = e3.symbol;
                s0 = e0.newState + bf_read(&f, e0.nbBits);
                s1 = e1.newState + bf_read(&f, e1.nbBits);
                s2 = e2.newState + bf_read(&f, e2.nbBits);
                s3 = e3.newState + bf_read(&f, e3.nbBits);
                bf_refill(&f);
                i += 4;
            }
            st[0] = s0, st[1] = s1, st[2] = s2, st[3] = s3;
        } else {
            uint32_t s0 = st[0], s1 = st[1];
            while (i + 4 <= lastTransition && f.p - src >= 8) {
                FseD e0 = dt[s0], e1 = dt[s1];
                dst[i] = e0.symbol;
                dst[i + 1] = e1.symbol;
                s0 = e0.newState + bf_read(&f, e0.nbBits);
                s1 = e1.newState + bf_read(&f, e1.nbBits);
                e0 = dt[s0], e1 = dt[s1];
                dst[i + 2] = e0.symbol;
                dst[i + 3] = e1.symbol;
                s0 = e0.newState + bf_read(&f, e0.nbBits);
                s1 = e1.newState + bf_read(&f, e1.nbBits);
                bf_refill(&f);
                i += 4;
            }
            st[0] = s0, st[1] = s1;
        }
        bc_at(&r, src, srcSize, bf_pos(&f, src));
    }
    /* i is a multiple of nbStates here: state k produces symbols i = k mod nbStates */
    for (unsigned k = 0; i < dstSize; i++) {
        FseD const e = dt[st[k]];
        dst[i] = e.symbol;
        if (i < lastTransition) {
            st[k] = e.newState + bc_peek(&r, e.nbBits);
            bc_skip(&r, e.nbBits);
        }
        if (++k == nbStates) k = 0;
    }
    if (r.pos != 0) return -OZO_ERR_CORRUPTION;
    return 0;
}

/* ---------------------------------------------------------------------
 * Huffman: weights -> canonical decoding table
 * (src/openzl/codecs/entropy/decode_entropy_binding.c:205-284,
 * src/openzl/fse/decompress/huf_decompress.c:342-454). Symbols are ranked by
 * weight then by value; a symbol of weight w spans 2^(w-1) cells and codes
 * on tableLog+1-w bits.
 * ------------------------------------------------------------------- */
typedef struct {
    uint8_t symbol;
    uint8_t nbBits;
} HufD;

static int huf_build_dtable(HufD* dt, unsigned* tableLogOut, const uint8_t* weights, size_t nbWeights)
{
    if (nbWeights < 2 || nbWeights > 256) return -1;
    uint32_t sum = 0;
    unsigned counts[16] = { 0 };
    for (size_t i = 0; i < nbWeights; i++) {
        if (weights[i] > 12) return -1;
        sum += (1u << weights[i]) >> 1;
        counts[weights[i]]++;
    }
    if (sum == 0 || (sum & (sum - 1))) return -1;
    unsigned const tableLog = (unsigned)ozo_highbit32(sum);
    if (tableLog > 12) return -1;
    if (nbWeights - counts[0] < 2) return -1;
    uint32_t pos = 0;
    for (unsigned w = 1; w <= tableLog; w++) {
        for (size_t s = 0; s < nbWeights; s++) {
            if (weights[s] != w) continue;
            uint32_t const len = (1u << w) >> 1;
            for (uint32_t u = 0; u < len; u++) {
                dt[pos + u].symbol = (uint8_t)s;
                dt[pos + u].nbBits = (uint8_t)(tableLog + 1 - w);
            }
            pos += len;
        }
    }
    *tableLogOut = tableLog;
    return 0;
}

/* The tail of one stream from symbol i on (the careful reader). */
static int huf_finish(uint8_t* dst, size_t i, size_t n, BCont* rp, const HufD* dt, unsigned tableLog)
{
    BCont r = *rp;
    for (; i < n; i++) {
        HufD const e = dt[bc_peek(&r, (int)tableLog)];
        dst[i] = e.symbol;
        bc_skip(&r, e.nbBits);
    }
    if (r.pos != 0) return -OZO_ERR_CORRUPTION;
    return 0;
}

static int huf_decode_stream(uint8_t* dst, size_t n, const uint8_t* src, size_t size,
                             const HufD* dt, unsigned tableLog)
{
    BCont r;
    if (bc_init(&r, src, size)) return -OZO_ERR_CORRUPTION;
    size_t i = 0;
    if (r.pos >= 64 && tableLog <= 12) { /* four codes (<= 48 bits) per refill */
        BFast f;
        bf_from(&f, src, r.pos);
        while (i + 4 <= n && f.p - src >= 8) {
            for (int k = 0; k < 4; k++) {
                HufD const e = dt[bf_peek(&f, tableLog)];
                dst[i + k] = e.symbol;
                f.used += e.nbBits;
            }
            bf_refill(&f);
            i += 4;
        }
        bc_at(&r, src, size, bf_pos(&f, src));
    }
    return huf_finish(dst, i, n, &r, dt, tableLog);
}

/* 4-stream layout: 6-byte jump table of three LE16 stream sizes, output split
 * into segments of (dstSize+3)/4 (src/openzl/fse/decompress/huf_decompress.c:
 * 562-660). */
static int huf_decode_4x(uint8_t* dst, size_t n, const uint8_t* src, size_t size,
                         const HufD* dt, unsigned tableLog)
{
    if (size < 10) return -OZO_ERR_CORRUPTION;
    size_t const l1 = ozo_rd16(src), l2 = ozo_rd16(src + 2), l3 = ozo_rd16(src + 4);
    if (l1 + l2 + l3 + 6 > size) return -OZO_ERR_CORRUPTION;
    size_t const l4 = size - 6 - l1 - l2 - l3;
    size_t const seg = (n + 3) / 4;
    if (3 * seg > n) return -OZO_ERR_CORRUPTION;
    const uint8_t* s = src + 6;
    const uint8_t* const ss[4] = { s, s + l1, s + l1 + l2, s + l1 + l2 + l3 };
    size_t const sz[4] = { l1, l2, l3, l4 };
    size_t const cnt[4] = { seg, seg, seg, n - 3 * seg };
    BCont r[4];
    for (int k = 0; k < 4; k++)
        if (bc_init(&r[k], ss[k], sz[k])) return -OZO_ERR_CORRUPTION;
    size_t i = 0;
    /* the four streams interleaved, four codes each per refill, while every
     * stream has room */
    if (tableLog <= 12 && r[0].pos >= 64 && r[1].pos >= 64 && r[2].pos >= 64 && r[3].pos >= 64) {
        BFast f[4];
        for (int k = 0; k < 4; k++) bf_from(&f[k], ss[k], r[k].pos);
        /* the four readers in locals: container, bits read, byte position */
        uint64_t c0 = f[0].c, c1 = f[1].c, c2 = f[2].c, c3 = f[3].c;
        unsigned u0 = f[0].used, u1 = f[1].used, u2 = f[2].used, u3 = f[3].used;
        const uint8_t *p0 = f[0].p, *p1 = f[1].p, *p2 = f[2].p, *p3 = f[3].p;
        const uint8_t *lo0 = ss[0] + 8, *lo1 = ss[1] + 8, *lo2 = ss[2] + 8, *lo3 = ss[3] + 8;
        unsigned const sh = 64 - tableLog;
        uint8_t* const o1 = dst + seg;
        uint8_t* const o2 = dst + 2 * seg;
        uint8_t* const o3 = dst + 3 * seg;
        while (i + 4 <= seg && p0 >= lo0 && p1 >= lo1 && p2 >= lo2 && p3 >= lo3) {
            for (int k = 0; k < 4; k++) {
                HufD const e0 = dt[(c0 << u0) >> sh];
                HufD const e1 = dt[(c1 << u1) >> sh];
                HufD const e2 = dt[(c2 << u2) >> sh];
                HufD const e3 = dt[(c3 << u3) >> sh];
                dst[i + k] = e0.symbol;
                o1[i + k] = e1.symbol;
                o2[i + k] = e2.symbol;
                o3[i + k] = e3.symbol;
                u0 += e0.nbBits;
                u1 += e1.nbBits;
                u2 += e2.nbBits;
                u3 += e3.nbBits;
            }
            p0 -= u0 >> 3, u0 &= 7, c0 = le64_at(p0);
            p1 -= u1 >> 3, u1 &= 7, c1 = le64_at(p1);
            p2 -= u2 >> 3, u2 &= 7, c2 = le64_at(p2);
            p3 -= u3 >> 3, u3 &= 7, c3 = le64_at(p3);
            i += 4;
        }
        f[0].c = c0, f[1].c = c1, f[2].c = c2, f[3].c = c3;
        f[0].used = u0, f[1].used = u1, f[2].used = u2, f[3].used = u3;
        f[0].p = p0, f[1].p = p1, f[2].p = p2, f[3].p = p3;
        for (int k = 0; k < 4; k++) bc_at(&r[k], ss[k], sz[k], bf_pos(&f[k], ss[k]));
    }
    for (int k = 0; k < 4; k++) {
        size_t const from = i < cnt[k] ? i : cnt[k];
        int const rc = huf_finish(dst + k * seg, from, cnt[k], &r[k], dt, tableLog);
        if (rc) return rc;
    }
    return 0;
}

/* ---------------------------------------------------------------------
 * 16-bit-symbol Huffman (huffman_struct_v2,
 * src/openzl/codecs/entropy/decode_entropy_binding.c:349-467 and
 * src/openzl/codecs/entropy/decode_huffman_kernel.c:35-290). Up to 65536
 * weights, at least two non-zero, weights and tableLog at most 20, the sum
 * of 2^(w-1) a power of two. Cells are ranked by weight (weight 1, the
 * longest code, first) then by symbol; a symbol of weight w spans 2^(w-1)
 * cells and codes on tableLog+1-w bits. The bitstream holds one stream, or
 * four in sequence, each prefixed by its symbol count and its byte size
 * (LE32 each); the streams together must fill the input exactly.
 * ------------------------------------------------------------------- */
typedef struct {
    uint16_t symbol;
    uint8_t nbBits;
} Huf16D;

static int huf16_build_dtable(Huf16D** dtOut, unsigned* tableLogOut, const uint8_t* weights, size_t nbWeights)
{
    if (nbWeights < 2 || nbWeights > 65536) return -1;
    size_t nz = 0;
    uint64_t sum = 0;
    unsigned counts[21] = { 0 };
    for (size_t i = 0; i < nbWeights; i++) {
        if (weights[i] > 20) return -1;
        nz += weights[i] != 0;
        sum += ((uint64_t)1 << weights[i]) >> 1;
        counts[weights[i]]++;
    }
    if (nz < 2 || sum == 0 || (sum & (sum - 1))) return -1;
    unsigned tableLog = 0;
    while (((uint64_t)1 << (tableLog + 1)) <= sum) tableLog++;
    if (tableLog > 20) return -1;
    Huf16D* dt = (Huf16D*)malloc(sizeof(Huf16D) << tableLog);
    if (!dt) return -1;
    size_t start[22];
    size_t pos = 0;
    for (unsigned w = 1; w <= tableLog; w++) {
        start[w] = pos;
        pos += (size_t)counts[w] << (w - 1);
    }
    for (size_t s = 0; s < nbWeights; s++) {
        unsigned const w = weights[s];
        if (!w) continue;
        size_t const len = (size_t)1 << (w - 1);
        for (size_t u = 0; u < len; u++) {
            dt[start[w] + u].symbol = (uint16_t)s;
            dt[start[w] + u].nbBits = (uint8_t)(tableLog + 1 - w);
        }
        start[w] += len;
    }
    *dtOut = dt;
    *tableLogOut = tableLog;
    return 0;
}

/* one stream: symbol count and byte size (LE32 each), then the backward
 * bitstream; decodes its symbols as 16-bit little-endian values */
static int huf16_decode_stream(uint8_t* dst, size_t cap, size_t* done, const uint8_t** src, size_t* avail,
                               const Huf16D* dt, unsigned tableLog)
{
    if (*avail < 8) return -OZO_ERR_CORRUPTION;
    size_t const n = ozo_rd32(*src), size = ozo_rd32(*src + 4);
    *src += 8;
    *avail -= 8;
    if (size > *avail || *done + n > cap) return -OZO_ERR_CORRUPTION;
    BCont r;
    if (bc_init(&r, *src, size)) return -OZO_ERR_CORRUPTION;
    for (size_t i = 0; i < n; i++) {
        Huf16D const e = dt[bc_peek(&r, (int)tableLog)];
        ozo_wr16(dst + 2 * (*done + i), e.symbol);
        bc_skip(&r, e.nbBits);
    }
    *src += size;
    *avail -= size;
    *done += n;
    return 0;
}

/* ---------------------------------------------------------------------
 * Decoder signatures (src/openzl/codecs/decoder_registry.c:88-161 and the
 * graph macros it names): number of singleton inputs with their types,
 * whether variable inputs are accepted, and the regenerated type.
 * ------------------------------------------------------------------- */
typedef struct {
    int known;
    int nbSO;
    int soTypes[2];
    int voType;   /* 0 when the decoder takes no variable inputs */
    int outType;  /* type of the regenerated stream */
} DecSig;

static DecSig sig_of(unsigned id)
{
    DecSig d = { 0 };
    d.known = 1;
    switch (id) {
        case TR_DELTA_INT:
        case TR_ZIGZAG:
            d.nbSO = 1; d.soTypes[0] = OZO_TYPE_NUMERIC; d.outType = OZO_TYPE_NUMERIC; break;
        case TR_TRANSPOSE_SPLIT:
            d.nbSO = 0; d.voType = OZO_TYPE_SERIAL; d.outType = OZO_TYPE_STRUCT; break;
        case TR_CONV_SERIAL_TO_STRUCT:
            d.nbSO = 1; d.soTypes[0] = OZO_TYPE_STRUCT; d.outType = OZO_TYPE_SERIAL; break;
        case TR_CONV_STRUCT_TO_SERIAL:
            d.nbSO = 1; d.soTypes[0] = OZO_TYPE_SERIAL; d.outType = OZO_TYPE_STRUCT; break;
        case TR_CONV_STRUCT_TO_NUM_LE:
            d.nbSO = 1; d.soTypes[0] = OZO_TYPE_NUMERIC; d.outType = OZO_TYPE_STRUCT; break;
        case TR_CONV_NUM_TO_STRUCT_LE:
            d.nbSO = 1; d.soTypes[0] = OZO_TYPE_STRUCT; d.outType = OZO_TYPE_NUMERIC; break;
        case TR_CONV_SERIAL_TO_NUM_LE:
            d.nbSO = 1; d.soTypes[0] = OZO_TYPE_NUMERIC; d.outType = OZO_TYPE_SERIAL; break;
        case TR_CONV_NUM_TO_SERIAL_LE:
            d.nbSO = 1; d.soTypes[0] = OZO_TYPE_SERIAL; d.outType = OZO_TYPE_NUMERIC; break;
        case TR_BITPACK_SERIAL:
            d.nbSO = 1; d.soTypes[0] = OZO_TYPE_SERIAL; d.outType = OZO_TYPE_SERIAL; break;
        case TR_BITPACK_INT:
            d.nbSO = 1; d.soTypes[0] = OZO_TYPE_SERIAL; d.outType = OZO_TYPE_NUMERIC; break;
        case TR_FLATPACK:
            d.nbSO = 2; d.soTypes[0] = OZO_TYPE_SERIAL; d.soTypes[1] = OZO_TYPE_SERIAL;
            d.outType = OZO_TYPE_SERIAL; break;
        case TR_FLOAT_DECONSTRUCT:
            d.nbSO = 2; d.soTypes[0] = OZO_TYPE_STRUCT; d.soTypes[1] = OZO_TYPE_SERIAL;
            d.outType = OZO_TYPE_NUMERIC; break;
        case TR_TOKENIZE_FIXED:
            d.nbSO = 2; d.soTypes[0] = OZO_TYPE_STRUCT; d.soTypes[1] = OZO_TYPE_NUMERIC;
            d.outType = OZO_TYPE_STRUCT; break;
        case TR_TOKENIZE_NUMERIC:
            d.nbSO = 2; d.soTypes[0] = OZO_TYPE_NUMERIC; d.soTypes[1] = OZO_TYPE_NUMERIC;
            d.outType = OZO_TYPE_NUMERIC; break;
        case TR_SPLITN:
            d.nbSO = 0; d.voType = OZO_TYPE_SERIAL; d.outType = OZO_TYPE_SERIAL; break;
        case TR_SPLITN_STRUCT:
            d.nbSO = 0; d.voType = OZO_TYPE_STRUCT; d.outType = OZO_TYPE_STRUCT; break;
        case TR_SPLITN_NUM:
            d.nbSO = 0; d.voType = OZO_TYPE_NUMERIC; d.outType = OZO_TYPE_NUMERIC; break;
        case TR_CONSTANT_SERIAL:
            d.nbSO = 1; d.soTypes[0] = OZO_TYPE_SERIAL; d.outType = OZO_TYPE_SERIAL; break;
        case TR_SEPARATE_STRING: /* graph_conversion.h:61-66, decoder inputs: content, lengths */
            d.nbSO = 2; d.soTypes[0] = OZO_TYPE_SERIAL; d.soTypes[1] = OZO_TYPE_NUMERIC;
            d.outType = OZO_TYPE_STRING; break;
        case TR_CONSTANT_FIXED:
            d.nbSO = 1; d.soTypes[0] = OZO_TYPE_STRUCT; d.outType = OZO_TYPE_STRUCT; break;
        case TR_FSE_V2:
        case TR_HUFFMAN_V2:
            d.nbSO = 2; d.soTypes[0] = OZO_TYPE_NUMERIC; d.soTypes[1] = OZO_TYPE_SERIAL;
            d.outType = OZO_TYPE_SERIAL; break;
        case TR_HUFFMAN_STRUCT_V2:
            d.nbSO = 2; d.soTypes[0] = OZO_TYPE_NUMERIC; d.soTypes[1] = OZO_TYPE_SERIAL;
            d.outType = OZO_TYPE_STRUCT; break;
        case TR_FSE_NCOUNT:
            d.nbSO = 1; d.soTypes[0] = OZO_TYPE_SERIAL; d.outType = OZO_TYPE_NUMERIC; break;
        default:
            d.known = 0;
    }
    return d;
}

/* ---------------------------------------------------------------------
 * Decoders. `in` holds the decoder's inputs in the decoder's own order
 * (src/openzl/decompress/decompress2.c:1132-1138 reverses stream slots).
 * ------------------------------------------------------------------- */
static int dec_run(unsigned id, OStream** in, size_t nbIn, const uint8_t* hdr, size_t hsz,
                   OStream* out)
{
    DecSig const sg = sig_of(id);
    switch (id) {
        case TR_SEPARATE_STRING: { /* DI_revert_VSF_separation, decode_conversion_binding.c:230-275 */
            const OStream* c = in[0];
            const OStream* l = in[1];
            size_t const nb = l->n;
            uint32_t* lens = (uint32_t*)malloc(nb * 4 + 4);
            uint64_t sum = 0;
            for (size_t i = 0; i < nb; i++) {
                uint64_t const v = ozo_rdN(l->p + i * l->w, l->w);
                if (v > 0xFFFFFFFFu) { free(lens); return -OZO_ERR_CORRUPTION; }
                lens[i] = (uint32_t)v;
                sum += v;
            }
            if (sum != (uint64_t)c->n * c->w) { free(lens); return -OZO_ERR_CORRUPTION; }
            ost_ref(out, OZO_TYPE_STRING, 1, c->n * c->w, c->p);
            out->lens = lens;
            out->nbStrings = nb;
            return 0;
        }
        case TR_DELTA_INT: { /* decode_delta_binding.c:11-58 */
            size_t const w = in[0]->w, nd = in[0]->n;
            size_t n = 0;
            if (hsz) {
                if (hsz != w) return -OZO_ERR_CORRUPTION;
                n = nd + 1;
            } else if (nd) {
                return -OZO_ERR_CORRUPTION;
            }
            uint8_t* o = ost_alloc(out, OZO_TYPE_NUMERIC, w, n);
            if (n) {
                uint64_t const m = w == 8 ? ~0ull : ((1ull << (8 * w)) - 1);
                uint64_t v = ozo_rdN(hdr, w);
                const uint8_t* const d = in[0]->p;
#define OZO_DELTA_W(T)                                                            \
    {                                                                             \
        T acc = (T)v;                                                             \
        memcpy(o, &acc, sizeof(T));                                               \
        for (size_t i = 1; i < n; i++) {                                          \
            T x;                                                                  \
            memcpy(&x, d + (i - 1) * sizeof(T), sizeof(T));                       \
            acc = (T)(acc + x);                                                   \
            memcpy(o + i * sizeof(T), &acc, sizeof(T));                           \
        }                                                                         \
    }
                switch (w) {
                    case 1: OZO_DELTA_W(uint8_t) break;
                    case 2: OZO_DELTA_W(uint16_t) break;
                    case 4: OZO_DELTA_W(uint32_t) break;
                    case 8: OZO_DELTA_W(uint64_t) break;
                    default:
                        for (size_t i = 0; i < n; i++) {
                            if (i) v = (v + ozo_rdN(d + (i - 1) * w, w)) & m;
                            for (size_t b = 0; b < w; b++) o[i * w + b] = (uint8_t)(v >> (8 * b));
                        }
                }
#undef OZO_DELTA_W
            }
            return 0;
        }
        case TR_ZIGZAG: { /* decode_zigzag_kernel.c */
            size_t const w = in[0]->w, n = in[0]->n;
            uint8_t* o = ost_alloc(out, OZO_TYPE_NUMERIC, w, n);
            uint64_t const m = w == 8 ? ~0ull : ((1ull << (8 * w)) - 1);
            for (size_t i = 0; i < n; i++) {
                uint64_t z = ozo_rdN(in[0]->p + i * w, w);
                uint64_t v = ((z >> 1) ^ (0 - (z & 1))) & m;
                for (size_t b = 0; b < w; b++) o[i * w + b] = (uint8_t)(v >> (8 * b));
            }
            return 0;
        }
        case TR_TRANSPOSE_SPLIT: { /* decode_transpose_binding.c:37-75 */
            if (nbIn == 0) return -OZO_ERR_CORRUPTION;
            size_t const n = in[0]->n, W = nbIn;
            for (size_t i = 0; i < nbIn; i++)
                if (in[i]->type != OZO_TYPE_SERIAL || in[i]->n != n) return -OZO_ERR_CORRUPTION;
            uint8_t* o = ost_alloc(out, OZO_TYPE_STRUCT, W, n);
            if (W == 2 || W == 4 || W == 8) { /* element-major: one pass over the output */
                const uint8_t* pl[8];
                for (size_t b = 0; b < W; b++) pl[b] = in[b]->p;
                /* the plane count as a constant, so the gather unrolls */
#define OZO_TSPLIT_W(NW, WR)                                                   \
    for (size_t e = 0; e < n; e++) {                                          \
        uint64_t v = 0;                                                       \
        for (size_t b = 0; b < (NW); b++) v |= (uint64_t)pl[b][e] << (8 * b); \
        WR;                                                                   \
    }
                if (W == 2) OZO_TSPLIT_W(2, ozo_wr16(o + 2 * e, (uint16_t)v))
                else if (W == 4) OZO_TSPLIT_W(4, ozo_wr32(o + 4 * e, (uint32_t)v))
                else OZO_TSPLIT_W(8, ozo_wr64(o + 8 * e, v))
#undef OZO_TSPLIT_W
                return 0;
            }
            for (size_t b = 0; b < W; b++) {
                const uint8_t* const pl = in[b]->p;
                uint8_t* const ob = o + b;
                for (size_t e = 0; e < n; e++) ob[e * W] = pl[e];
            }
            return 0;
        }
        case TR_CONV_NUM_TO_STRUCT_LE: { /* decode_conversion_binding.c:190-225 */
            size_t const w = in[0]->w;
            if (!(w == 1 || w == 2 || w == 4 || w == 8)) return -OZO_ERR_CORRUPTION;
            ost_ref(out, OZO_TYPE_NUMERIC, w, in[0]->n, in[0]->p);
            return 0;
        }
        case TR_CONV_STRUCT_TO_NUM_LE: /* decode_conversion_binding.c:178-188 */
            ost_ref(out, OZO_TYPE_STRUCT, in[0]->w, in[0]->n, in[0]->p);
            return 0;
        case TR_CONV_SERIAL_TO_NUM_LE: /* decode_conversion_binding.c:60-64 */
            ost_ref(out, OZO_TYPE_SERIAL, 1, in[0]->n * in[0]->w, in[0]->p);
            return 0;
        case TR_CONV_SERIAL_TO_STRUCT: /* decode_conversion_binding.c:112-122 */
            ost_ref(out, OZO_TYPE_SERIAL, 1, in[0]->n * in[0]->w, in[0]->p);
            return 0;
        case TR_CONV_NUM_TO_SERIAL_LE: { /* decode_conversion_binding.c:72-110 */
            if (hsz != 1) return -OZO_ERR_CORRUPTION;
            size_t const w = (size_t)1 << hdr[0];
            if (!(w == 1 || w == 2 || w == 4 || w == 8)) return -OZO_ERR_CORRUPTION;
            size_t const bytes = in[0]->n * in[0]->w;
            if (bytes % w) return -OZO_ERR_CORRUPTION;
            uint8_t* o = ost_alloc(out, OZO_TYPE_NUMERIC, w, bytes / w);
            memcpy(o, in[0]->p, bytes);
            return 0;
        }
        case TR_CONV_STRUCT_TO_SERIAL: { /* decode_conversion_binding.c:125-160 */
            const uint8_t* p = hdr;
            uint64_t ew;
            if (ozo_varint_dec(&p, hdr + hsz, &ew) || p != hdr + hsz || ew == 0) return -OZO_ERR_CORRUPTION;
            size_t const bytes = in[0]->n * in[0]->w;
            if (bytes % ew) return -OZO_ERR_CORRUPTION;
            ost_ref(out, OZO_TYPE_STRUCT, (size_t)ew, bytes / ew, in[0]->p);
            return 0;
        }
        case TR_BITPACK_SERIAL:
        case TR_BITPACK_INT: { /* decode_bitpack_binding.c:9-60 */
            if (hsz < 1 || hsz > 2) return -OZO_ERR_CORRUPTION;
            size_t const w = (size_t)1 << ((hdr[0] >> 6) & 3);
            int const nbBits = 1 + (hdr[0] & 0x3f);
            if ((size_t)nbBits > 8 * w) return -OZO_ERR_CORRUPTION;
            if (id == TR_BITPACK_SERIAL && w != 1) return -OZO_ERR_CORRUPTION;
            size_t const srcSize = in[0]->n;
            size_t const maxN = srcSize * 8 / (size_t)nbBits;
            size_t n = maxN;
            if (hsz > 1) {
                if (hdr[1] > maxN) return -OZO_ERR_CORRUPTION;
                n = maxN - hdr[1];
            }
            if ((n * (size_t)nbBits + 7) / 8 != srcSize) return -OZO_ERR_CORRUPTION;
            uint8_t* o = ost_alloc(out, sg.outType, w, n);
            const uint8_t* const src = in[0]->p;
            uint64_t const mask = nbBits >= 64 ? ~0ull : ((1ull << nbBits) - 1);
            /* bulk: fields whose 8-byte load stays inside the source and
             * holds the whole field; the rest through bitunpack */
            size_t i = 0;
            if ((size_t)nbBits == 8 * w) { /* whole elements: the packing is the identity */
                memcpy(o, src, n * w);
                i = n;
            } else if (nbBits > 56) { /* 57..63 bits: the field spans up to 9 bytes */
                size_t const fast = srcSize >= 9 ? ((srcSize - 9) * 8) / (size_t)nbBits : 0;
                size_t const m = fast < n ? fast : n;
                for (; i < m; i++) {
                    size_t const bit = i * (size_t)nbBits;
                    unsigned const sh = (unsigned)(bit & 7);
                    uint64_t v = le64_at(src + (bit >> 3)) >> sh;
                    if (sh) v |= (uint64_t)src[(bit >> 3) + 8] << (64 - sh);
                    ozo_wr64(o + 8 * i, v & mask);
                }
            } else {
                size_t const fast = srcSize >= 8 ? ((srcSize - 8) * 8) / (size_t)nbBits : 0;
                size_t const m = fast < n ? fast : n;
#define OZO_UNPACK_W(T, WR)                                                  \
    for (; i < m; i++) {                                                     \
        size_t const bit = i * (size_t)nbBits;                               \
        uint64_t const v = (le64_at(src + (bit >> 3)) >> (bit & 7)) & mask;  \
        WR;                                                                  \
    }
                switch (w) {
                    case 1: OZO_UNPACK_W(uint8_t, o[i] = (uint8_t)v) break;
                    case 2: OZO_UNPACK_W(uint16_t, ozo_wr16(o + 2 * i, (uint16_t)v)) break;
                    case 4: OZO_UNPACK_W(uint32_t, ozo_wr32(o + 4 * i, (uint32_t)v)) break;
                    default: OZO_UNPACK_W(uint64_t, ozo_wr64(o + 8 * i, v)) break;
                }
#undef OZO_UNPACK_W
            }
            for (; i < n; i++) { /* the last fields, bit by bit */
                size_t const bit = i * (size_t)nbBits;
                uint64_t v = 0;
                for (int q = 0; q < nbBits; q++) {
                    size_t const bq = bit + (size_t)q;
                    v |= (uint64_t)((src[bq >> 3] >> (bq & 7)) & 1) << q;
                }
                switch (w) {
                    case 1: o[i] = (uint8_t)v; break;
                    case 2: ozo_wr16(o + 2 * i, (uint16_t)v); break;
                    case 4: ozo_wr32(o + 4 * i, (uint32_t)v); break;
                    default: ozo_wr64(o + 8 * i, v); break;
                }
            }
            return 0;
        }
        case TR_FLATPACK: { /* decode_flatpack_binding.c, decode_flatpack_kernel.c:19-60 */
            const OStream* alpha = in[0];
            const OStream* packed = in[1];
            size_t const asz = alpha->n;
            if (asz > 256) return -OZO_ERR_CORRUPTION;
            size_t const psz = packed->n;
            size_t n = 0;
            unsigned nbBits = asz <= 1 ? (unsigned)asz : 1u + (unsigned)ozo_highbit32((uint32_t)asz - 1);
            if (psz && asz) {
                uint32_t last = packed->p[psz - 1] | 1;
                size_t pad = (size_t)__builtin_clz(last << 24) + 1;
                n = (8 * psz - pad) / nbBits;
            }
            uint8_t* o = ost_alloc(out, OZO_TYPE_SERIAL, 1, n);
            size_t bit = 0;
            /* an index of at most 8 bits lies in the two bytes from bit >> 3 */
            unsigned const mask = (1u << nbBits) - 1u;
            for (size_t i = 0; i < n; i++, bit += nbBits) {
                size_t const q = bit >> 3;
                unsigned const win = packed->p[q] | (q + 1 < psz ? (unsigned)packed->p[q + 1] << 8 : 0u);
                unsigned const idx = (win >> (bit & 7)) & mask;
                if (idx >= asz) return -OZO_ERR_CORRUPTION;
                o[i] = alpha->p[idx];
            }
            if (psz && asz) {
                /* terminator bit then zero padding */
                if (!((packed->p[bit >> 3] >> (bit & 7)) & 1)) return -OZO_ERR_CORRUPTION;
                if ((bit >> 3) != psz - 1) return -OZO_ERR_CORRUPTION;
            }
            return 0;
        }
        case TR_FLOAT_DECONSTRUCT: { /* decode_float_deconstruct_binding.c:13-70 */
            const OStream* sf = in[0];
            const OStream* ex = in[1];
            if (hsz != 1 || hdr[0] > 2) return -OZO_ERR_CORRUPTION;
            size_t const n = ex->n;
            if (sf->n != n) return -OZO_ERR_CORRUPTION;
            unsigned const t = hdr[0];
            size_t const sfw = t == 0 ? 3 : (t == 1 ? 1 : 2);
            if (sf->w != sfw || ex->w != 1) return -OZO_ERR_CORRUPTION;
            size_t const ow = t == 0 ? 4 : 2;
            uint8_t* o = ost_alloc(out, OZO_TYPE_NUMERIC, ow, n);
            for (size_t i = 0; i < n; i++) {
                if (t == 1) {
                    uint8_t s = sf->p[i];
                    uint16_t v = (uint16_t)((s >> 1) | ((uint16_t)s << 15) | ((uint16_t)ex->p[i] << 7));
                    ozo_wr16(o + 2 * i, v);
                } else if (t == 2) {
                    uint16_t s = ozo_rd16(sf->p + 2 * i);
                    uint16_t v = (uint16_t)((s >> 1) | (uint16_t)(s << 15) | ((uint16_t)ex->p[i] << 10));
                    ozo_wr16(o + 2 * i, v);
                } else {
                    uint32_t s = (uint32_t)ozo_rdN(sf->p + 3 * i, 3);
                    uint32_t v = ((uint32_t)ex->p[i] << 23) | (s << 31) | (s >> 1);
                    ozo_wr32(o + 4 * i, v);
                }
            }
            return 0;
        }
        case TR_TOKENIZE_FIXED:
        case TR_TOKENIZE_NUMERIC: { /* decode_tokenize_binding.c:9-38 */
            const OStream* alpha = in[0];
            const OStream* idx = in[1];
            size_t const w = alpha->w, n = idx->n, iw = idx->w;
            uint8_t* o = ost_alloc(out, sg.outType, w, n);
            for (size_t i = 0; i < n; i++) {
                uint64_t k = ozo_rdN(idx->p + i * iw, iw);
                if (k >= alpha->n) return -OZO_ERR_CORRUPTION;
                memcpy(o + i * w, alpha->p + k * w, w);
            }
            return 0;
        }
        case TR_SPLITN:
        case TR_SPLITN_STRUCT:
        case TR_SPLITN_NUM: { /* decode_splitN_binding.c:16-80 */
            size_t w = 1;
            int type = sg.outType;
            if (nbIn == 0) {
                if (hsz) {
                    const uint8_t* p = hdr;
                    uint64_t v;
                    if (ozo_varint_dec(&p, hdr + hsz, &v)) return -OZO_ERR_CORRUPTION;
                    w = (size_t)v;
                }
            } else {
                w = in[0]->w;
                type = in[0]->type;
            }
            size_t total = 0;
            for (size_t i = 0; i < nbIn; i++) {
                if (in[i]->type != type || in[i]->w != w) return -OZO_ERR_CORRUPTION;
                total += in[i]->n;
            }
            uint8_t* o = ost_alloc(out, sg.outType, w, total);
            size_t pos = 0;
            for (size_t i = 0; i < nbIn; i++) {
                memcpy(o + pos, in[i]->p, in[i]->n * w);
                pos += in[i]->n * w;
            }
            return 0;
        }
        case TR_CONSTANT_SERIAL:
        case TR_CONSTANT_FIXED: { /* decode_constant_binding.c:10-45 */
            if (in[0]->n != 1) return -OZO_ERR_CORRUPTION;
            const uint8_t* p = hdr;
            uint64_t n;
            if (ozo_varint_dec(&p, hdr + hsz, &n) || p != hdr + hsz || n < 1) return -OZO_ERR_CORRUPTION;
            size_t const w = in[0]->w;
            uint8_t* o = ost_alloc(out, sg.outType, w, (size_t)n);
            for (size_t i = 0; i < n; i++) memcpy(o + i * w, in[0]->p, w);
            return 0;
        }
        case TR_FSE_NCOUNT: { /* decode_entropy_binding.c:118-143 */
            int16_t norm[256];
            unsigned maxSV = 255, tl = 0;
            int64_t r = fse_read_ncount(norm, &maxSV, &tl, in[0]->p, in[0]->n);
            if (r < 0 || (size_t)r != in[0]->n) return -OZO_ERR_CORRUPTION;
            uint8_t* o = ost_alloc(out, OZO_TYPE_NUMERIC, 2, maxSV + 1);
            for (unsigned s = 0; s <= maxSV; s++) ozo_wr16(o + 2 * s, (uint16_t)norm[s]);
            return 0;
        }
        case TR_FSE_V2: { /* decode_entropy_binding.c:24-116 */
            const OStream* normS = in[0];
            const OStream* bits = in[1];
            if (normS->w != 2) return -OZO_ERR_CORRUPTION;
            size_t const nbSym = normS->n;
            if (nbSym < 2 || nbSym > 256) return -OZO_ERR_CORRUPTION;
            int16_t norm[256];
            unsigned sum = 0;
            for (size_t i = 0; i < nbSym; i++) {
                norm[i] = (int16_t)ozo_rd16(normS->p + 2 * i);
                if (norm[i] < -1) return -OZO_ERR_CORRUPTION;
                sum += norm[i] == -1 ? 1u : (unsigned)norm[i];
            }
            if (sum == 0 || (sum & (sum - 1))) return -OZO_ERR_CORRUPTION;
            unsigned const tl = (unsigned)ozo_highbit32(sum);
            if (tl < 5 || tl > 12) return -OZO_ERR_CORRUPTION;
            if (hsz < 2 || hsz > 9) return -OZO_ERR_CORRUPTION;
            unsigned const nbStates = hdr[0];
            if (nbStates != 2 && nbStates != 4) return -OZO_ERR_CORRUPTION;
            size_t const dstSize = (size_t)ozo_rdN(hdr + 1, hsz - 1);
            if (dstSize < 2) return -OZO_ERR_CORRUPTION;
            FseD* dt = (FseD*)malloc(sizeof(FseD) << tl);
            if (fse_build_dtable(dt, norm, (unsigned)nbSym - 1, tl)) { free(dt); return -OZO_ERR_CORRUPTION; }
            uint8_t* o = ost_alloc(out, OZO_TYPE_SERIAL, 1, dstSize);
            int rc = fse_decode(o, dstSize, bits->p, bits->n, dt, tl, nbStates);
            free(dt);
            return rc;
        }
        case TR_HUFFMAN_V2: { /* decode_entropy_binding.c:286-347 */
            const OStream* wS = in[0];
            const OStream* bits = in[1];
            if (wS->w != 1) return -OZO_ERR_CORRUPTION;
            if (hsz < 2 || hsz > 9) return -OZO_ERR_CORRUPTION;
            int const x4 = hdr[0] & 1;
            size_t const dstSize = (size_t)ozo_rdN(hdr + 1, hsz - 1);
            if (dstSize < 2) return -OZO_ERR_CORRUPTION;
            HufD dt[4096];
            unsigned tl;
            if (huf_build_dtable(dt, &tl, wS->p, wS->n)) return -OZO_ERR_CORRUPTION;
            uint8_t* o = ost_alloc(out, OZO_TYPE_SERIAL, 1, dstSize);
            return x4 ? huf_decode_4x(o, dstSize, bits->p, bits->n, dt, tl)
                      : huf_decode_stream(o, dstSize, bits->p, bits->n, dt, tl);
        }
        case TR_HUFFMAN_STRUCT_V2: { /* decode_entropy_binding.c:415-467 */
            const OStream* wS = in[0];
            const OStream* bits = in[1];
            if (wS->w != 1) return -OZO_ERR_CORRUPTION;
            if (hsz < 2 || hsz > 9) return -OZO_ERR_CORRUPTION;
            int const x4 = hdr[0] & 1;
            size_t const dstSize = (size_t)ozo_rdN(hdr + 1, hsz - 1);
            if (dstSize < 2) return -OZO_ERR_CORRUPTION;
            Huf16D* dt = NULL;
            unsigned tl;
            if (huf16_build_dtable(&dt, &tl, wS->p, wS->n)) return -OZO_ERR_CORRUPTION;
            uint8_t* o = ost_alloc(out, OZO_TYPE_STRUCT, 2, dstSize);
            const uint8_t* p = bits->p;
            size_t avail = bits->n, done = 0;
            int rc = 0;
            for (int k = 0; k < (x4 ? 4 : 1) && !rc; k++) rc = huf16_decode_stream(o, dstSize, &done, &p, &avail, dt, tl);
            free(dt);
            if (rc) return rc;
            if (done != dstSize || avail != 0) return -OZO_ERR_CORRUPTION;
            return 0;
        }
        default:
            return -OZO_ERR_UNSUPPORTED;
    }
}

/* ---------------------------------------------------------------------
 * Frame and block parsing, and the stream-slot executor
 * (src/openzl/decompress/decode_frameheader.c:237-340, 938-1171;
 * src/openzl/decompress/decompress2.c:632-834, 1046-1290, 1442-1570).
 * ------------------------------------------------------------------- */
#define OZO_MAX_OUTPUTS 64

typedef struct {
    unsigned version;
    int hasContentCk, hasCompressedCk;
    size_t nbOutputs;
    int types[OZO_MAX_OUTPUTS];
    uint64_t sizes[OZO_MAX_OUTPUTS];
    uint64_t nbStrings[OZO_MAX_OUTPUTS]; /* string outputs, v21+ */
    size_t headerSize;
} FrameHdr;

static int decode_type(unsigned t)
{
    static const int m[4] = { OZO_TYPE_SERIAL, OZO_TYPE_STRUCT, OZO_TYPE_NUMERIC, OZO_TYPE_STRING };
    return m[t & 3];
}

/* Frame header of format versions 8..20: no flags byte (the checksum flags
 * sit in the chunk header), the output count and types packed into byte 4
 * onwards, sizes as LE32, no comment, no header checksum
 * (decode_frameheader.c:58-92 count, 110-147 types, 177-190 sizes). */
static int64_t parse_frame_header_v20(FrameHdr* fh, const uint8_t* src, size_t size)
{
    unsigned const v = fh->version;
    size_t pos = 4, nbOut = 1;
    if (v >= 15) {
        if (size < pos + 1 + 4) return -OZO_ERR_SRC_SIZE;
        nbOut = (size_t)(src[pos++] >> 6) + 1;
        if (nbOut == 4) {
            if (pos >= size) return -OZO_ERR_SRC_SIZE;
            nbOut = (size_t)(src[pos++] >> 4) + 4;
        }
        if (nbOut == 19) {
            if (pos >= size) return -OZO_ERR_SRC_SIZE;
            nbOut = (size_t)src[pos++] + 19;
        }
        if (nbOut == 274) {
            if (pos + 2 > size) return -OZO_ERR_SRC_SIZE;
            nbOut = (size_t)ozo_rd16(src + pos) + 274;
            pos += 2;
        }
    } else if (v == 14) {
        pos++; /* the type byte */
    }
    if (nbOut > OZO_MAX_OUTPUTS) return -OZO_ERR_UNSUPPORTED;
    fh->nbOutputs = nbOut;
    if (v < 14) {
        fh->types[0] = OZO_TYPE_SERIAL;
    } else {
        if (size < 5) return -OZO_ERR_SRC_SIZE;
        for (size_t n = 0; n < nbOut && n < 3; n++) fh->types[n] = decode_type(src[4] >> (2 * n));
        if (nbOut > 3) {
            if (size < 6) return -OZO_ERR_SRC_SIZE;
            for (size_t n = 3; n < nbOut && n < 5; n++) fh->types[n] = decode_type(src[5] >> (2 * (n - 3)));
        }
        uint8_t tok = 0;
        for (size_t n = 5; n < nbOut; n++) {
            size_t const sh = ((n - 5) % 4) * 2;
            if (sh == 0) {
                if (pos >= size) return -OZO_ERR_SRC_SIZE;
                tok = src[pos++];
            }
            fh->types[n] = decode_type(tok >> sh);
        }
    }
    if (pos + 4 * nbOut > size) return -OZO_ERR_SRC_SIZE;
    for (size_t n = 0; n < nbOut; n++) fh->sizes[n] = ozo_rd32(src + pos + 4 * n);
    pos += 4 * nbOut;
    fh->headerSize = pos;
    return (int64_t)pos;
}

static int64_t parse_frame_header(FrameHdr* fh, const uint8_t* src, size_t size)
{
    memset(fh, 0, sizeof(*fh));
    if (size < 9) return -OZO_ERR_SRC_SIZE;
    uint32_t const magic = ozo_rd32(src);
    /* ZL_MIN_FORMAT_VERSION .. ZL_MAX_FORMAT_VERSION (openzl/zl_version.h) */
    if (magic < OZO_MAGIC_BASE + 8 || magic > OZO_MAGIC_BASE + 23) return -OZO_ERR_VERSION;
    fh->version = magic - OZO_MAGIC_BASE;
    if (fh->version < 21) return parse_frame_header_v20(fh, src, size);
    size_t pos = 4;
    uint8_t const flags = src[pos++];
    fh->hasContentCk = flags & 1;
    fh->hasCompressedCk = (flags >> 1) & 1;
    int const hasComment = (flags >> 2) & 1;
    /* output count and types (decode_frameheader.c:94-107, 148-173): up to
     * 14 outputs in the low nibble with the first two types above it, else
     * an extension byte and all types in the following bytes */
    uint8_t const t1 = src[pos++];
    size_t nbOut = t1 & 15;
    size_t done = 0;
    if (nbOut == 15) {
        if (pos >= size) return -OZO_ERR_SRC_SIZE;
        nbOut = ((size_t)src[pos++] << 4) + (t1 >> 4) + 15;
    } else {
        for (size_t n = 0; n < nbOut && n < 2; n++) fh->types[n] = decode_type(t1 >> (4 + 2 * n));
        done = 2;
    }
    if (nbOut == 0) return -OZO_ERR_UNSUPPORTED;
    if (nbOut > OZO_MAX_OUTPUTS) return -OZO_ERR_UNSUPPORTED;
    fh->nbOutputs = nbOut;
    if (nbOut > done) {
        uint8_t tok = 0;
        for (size_t n = done; n < nbOut; n++) {
            size_t const sh = ((n - done) % 4) * 2;
            if (sh == 0) {
                if (pos >= size) return -OZO_ERR_SRC_SIZE;
                tok = src[pos++];
            }
            fh->types[n] = decode_type(tok >> sh);
        }
    }
    const uint8_t* p = src + pos;
    if (*p == 0) return -OZO_ERR_UNSUPPORTED; /* unknown sizes */
    for (size_t n = 0; n < nbOut; n++) {
        uint64_t v;
        if (ozo_varint_dec(&p, src + size, &v) || v == 0) return -OZO_ERR_CORRUPTION;
        fh->sizes[n] = v - 1;
    }
    /* string outputs: their string counts follow (decode_frameheader.c:217-236) */
    for (size_t n = 0; n < nbOut; n++)
        if (fh->types[n] == OZO_TYPE_STRING && ozo_varint_dec(&p, src + size, &fh->nbStrings[n])) return -OZO_ERR_CORRUPTION;
    pos = (size_t)(p - src);
    if (fh->version >= 22 && hasComment) {
        uint64_t csz;
        if (ozo_varint_dec(&p, src + size, &csz) || csz == 0) return -OZO_ERR_CORRUPTION;
        pos = (size_t)(p - src) + (size_t)csz;
        if (pos > size) return -OZO_ERR_SRC_SIZE;
    }
    if (fh->hasCompressedCk) {
        if (pos + 1 > size) return -OZO_ERR_SRC_SIZE;
        if ((ozo_xxh3_64(src, pos) & 255) != src[pos]) return -OZO_ERR_CHECKSUM;
        pos++;
    }
    fh->headerSize = pos;
    return (int64_t)pos;
}

typedef struct {
    unsigned id;
    size_t hdrStart, hdrSize;
    size_t nbVOs, nbRegens;
    uint32_t* dist;
} DNode;

/* Decodes one block; appends each output to outs[]. Returns block size. */
static int64_t decode_block(const FrameHdr* fh, const uint8_t* src, size_t size, size_t start,
                            uint8_t** outBuf, size_t* outLen, int* outType, size_t* outW, uint32_t** outLens,
                            size_t* outNbStrings)
{
    const uint8_t* p = src + start;
    const uint8_t* const end = src + size;
    unsigned const ver = fh->version;
    uint64_t nbDec, nbStored;
    /* counts: single bytes before v9, varints after; the decoder count is
     * stored +1 from v21 (decode_frameheader.c:954-972) */
    if (ver < 9) {
        if (end - p < 2) return -OZO_ERR_SRC_SIZE;
        nbDec = p[0];
        nbStored = p[1];
        p += 2;
    } else {
        if (ozo_varint_dec(&p, end, &nbDec)) return -OZO_ERR_CORRUPTION;
        if (ver >= 21) {
            if (nbDec == 0) return -OZO_ERR_CORRUPTION;
            nbDec--;
        }
        if (ozo_varint_dec(&p, end, &nbStored)) return -OZO_ERR_CORRUPTION;
    }
    /* ZL_runtimeNodeLimit / ZL_runtimeStreamLimit (common/limits.c:18-46) */
    uint64_t const nodeLimit = ver < 9 ? 256 : ver < 20 ? 10000 : 20000;
    uint64_t const streamLimit = ver < 9 ? 256 : ver < 16 ? 10000 : 110000;
    if (nbDec >= nodeLimit || nbStored >= streamLimit) return -OZO_ERR_CORRUPTION;
    /* before v21 the checksum flags open the chunk header
     * (decode_frameheader.c:1002-1011) */
    int hasContentCk = fh->hasContentCk, hasCompressedCk = fh->hasCompressedCk;
    if (ver < 21) {
        if (p >= end) return -OZO_ERR_SRC_SIZE;
        hasContentCk = p[0] & 1;
        hasCompressedCk = (p[0] >> 1) & 1;
        p++;
    }
    size_t const nd = (size_t)nbDec, ns = (size_t)nbStored;
    DNode* nodes = (DNode*)calloc(nd + 1, sizeof(DNode));
    uint64_t* tmp = (uint64_t*)calloc(nd + ns + 8, 8);
    uint8_t* trt = (uint8_t*)calloc(nd + 1, 1);
    size_t* storedSizes = (size_t*)calloc(ns + 1, sizeof(size_t));
    uint32_t* dists = NULL;
    OStream* streams = NULL;
    int64_t ret = 0;
    OStream** insHeap = NULL; /* decoder input lists longer than 300 */
    size_t insHeapCap = 0;
#define FAIL(code) do { ret = -(code); goto done; } while (0)
    size_t r;
    /* codec types: 1 bit each */
    r = bitunpack(tmp, nd, p, (size_t)(end - p), 1);
    if (r == (size_t)-1) FAIL(OZO_ERR_SRC_SIZE);
    p += r;
    size_t nbStd = 0;
    for (size_t u = 0; u < nd; u++) { trt[u] = (uint8_t)tmp[u]; nbStd += !tmp[u]; }
    if (nbStd != nd) FAIL(OZO_ERR_UNSUPPORTED); /* custom codecs */
    /* standard IDs: nextPow2(63) = 6 bits each */
    r = bitunpack(tmp, nd, p, (size_t)(end - p), ozo_nextpow2(TR_END));
    if (r == (size_t)-1) FAIL(OZO_ERR_SRC_SIZE);
    p += r;
    for (size_t u = 0; u < nd; u++) nodes[u].id = (unsigned)tmp[u];
    /* codec header sizes: 1-bit non-zero flags, then varint(size-1) */
    r = bitunpack(tmp, nd, p, (size_t)(end - p), 1);
    if (r == (size_t)-1) FAIL(OZO_ERR_SRC_SIZE);
    p += r;
    size_t totalTH = 0;
    for (size_t u = 0; u < nd; u++) {
        size_t hs = 0;
        if (tmp[u]) {
            uint64_t v;
            if (ozo_varint_dec(&p, end, &v)) FAIL(OZO_ERR_CORRUPTION);
            hs = (size_t)v + 1;
        }
        nodes[u].hdrStart = totalTH;
        nodes[u].hdrSize = hs;
        totalTH += hs;
    }
    /* number of variable inputs: 1-bit flags, then varint(n-1) */
    r = bitunpack(tmp, nd, p, (size_t)(end - p), 1);
    if (r == (size_t)-1) FAIL(OZO_ERR_SRC_SIZE);
    p += r;
    for (size_t u = 0; u < nd; u++) {
        nodes[u].nbVOs = 0;
        if (tmp[u]) {
            uint64_t v;
            if (ozo_varint_dec(&p, end, &v)) FAIL(OZO_ERR_CORRUPTION);
            nodes[u].nbVOs = (size_t)v + 1;
        }
    }
    /* number of regenerated streams: 1-bit flags, then varint(n-2); every
     * decoder regenerates one stream before v16 (decode_frameheader.c:1068-1082) */
    if (ver >= 16) {
        r = bitunpack(tmp, nd, p, (size_t)(end - p), 1);
        if (r == (size_t)-1) FAIL(OZO_ERR_SRC_SIZE);
        p += r;
    } else {
        memset(tmp, 0, nd * sizeof(tmp[0]));
    }
    size_t totalRegens = 0;
    for (size_t u = 0; u < nd; u++) {
        nodes[u].nbRegens = 1;
        if (tmp[u]) {
            uint64_t v;
            if (ozo_varint_dec(&p, end, &v)) FAIL(OZO_ERR_CORRUPTION);
            nodes[u].nbRegens = (size_t)v + 2;
        }
        totalRegens += nodes[u].nbRegens;
    }
    /* regenerated-stream distances */
    dists = (uint32_t*)calloc(totalRegens + 1, 4);
    {
        uint64_t* dt = (uint64_t*)calloc(totalRegens + 1, 8);
        r = bitunpack(dt, totalRegens, p, (size_t)(end - p), ozo_nextpow2(totalRegens + ns));
        if (r == (size_t)-1) { free(dt); FAIL(OZO_ERR_SRC_SIZE); }
        p += r;
        for (size_t i = 0; i < totalRegens; i++) dists[i] = (uint32_t)dt[i];
        free(dt);
    }
    for (size_t u = 0, d = 0; u < nd; u++) { nodes[u].dist = dists + d; d += nodes[u].nbRegens; }
    /* stored stream sizes */
    for (size_t u = 0; u < ns; u++) {
        uint64_t v;
        if (ozo_varint_dec(&p, end, &v) || v >= 0xFFFFFFFFu) FAIL(OZO_ERR_CORRUPTION);
        storedSizes[u] = (size_t)v;
    }
    /* stream slots: regenerated ones marked, the rest filled from storage */
    {
        size_t const total = ns + totalRegens;
        size_t const firstOutput = total - fh->nbOutputs;
        streams = (OStream*)calloc(total + 1, sizeof(OStream));
        uint8_t* isRegen = (uint8_t*)calloc(total + 1, 1);
        size_t sidx = 0;
        for (size_t u = 0; u < nd; u++) {
            DecSig const sg = sig_of(nodes[u].id);
            if (!sg.known) { free(isRegen); FAIL(OZO_ERR_UNSUPPORTED); }
            if (!sg.voType && nodes[u].nbVOs) { free(isRegen); FAIL(OZO_ERR_CORRUPTION); }
            size_t const inEnd = sidx + (size_t)sg.nbSO + nodes[u].nbVOs;
            if (inEnd > firstOutput) { free(isRegen); FAIL(OZO_ERR_CORRUPTION); }
            for (size_t k = 0; k < nodes[u].nbRegens; k++) {
                size_t const o = inEnd + nodes[u].dist[k];
                if (o >= total || isRegen[o]) { free(isRegen); FAIL(OZO_ERR_CORRUPTION); }
                isRegen[o] = 1;
            }
            sidx = inEnd;
        }
        size_t pos = (size_t)(p - src);
        size_t const thStart = pos;
        pos += totalTH;
        if (pos > size) { free(isRegen); FAIL(OZO_ERR_SRC_SIZE); }
        size_t st = 0;
        for (size_t i = 0; i < total; i++) {
            if (isRegen[i]) continue;
            if (st == ns) { free(isRegen); FAIL(OZO_ERR_CORRUPTION); }
            if (pos + storedSizes[st] > size) { free(isRegen); FAIL(OZO_ERR_SRC_SIZE); }
            ost_ref(&streams[i], OZO_TYPE_SERIAL, 1, storedSizes[st], src + pos);
            pos += storedSizes[st];
            st++;
        }
        free(isRegen);
        if (st != ns) FAIL(OZO_ERR_CORRUPTION);
        uint32_t contentCk = 0;
        if (hasContentCk) {
            if (pos + 4 > size) FAIL(OZO_ERR_SRC_SIZE);
            contentCk = ozo_rd32(src + pos);
            pos += 4;
        }
        if (hasCompressedCk) {
            /* versions before 21 hash the frame from its first byte, later
             * ones the current block only (decompress2.c:1494-1500) */
            size_t const hs = ver < 21 ? 0 : start;
            if (pos + 4 > size) FAIL(OZO_ERR_SRC_SIZE);
            uint32_t const want = ozo_rd32(src + pos);
            if ((uint32_t)ozo_xxh3_64(src + hs, pos - hs) != want) FAIL(OZO_ERR_CHECKSUM);
            pos += 4;
        }
        /* run decoders in order */
        sidx = 0;
        for (size_t u = 0; u < nd; u++) {
            DecSig const sg = sig_of(nodes[u].id);
            size_t const nbIn = (size_t)sg.nbSO + nodes[u].nbVOs;
            OStream* insFixed[300];
            OStream** ins = insFixed;
            if (nbIn > 300) { /* concatenations of many chunks */
                if (nbIn > insHeapCap) {
                    OStream** g = (OStream**)realloc(insHeap, nbIn * sizeof(OStream*));
                    if (!g) FAIL(OZO_ERR_ALLOC);
                    insHeap = g;
                    insHeapCap = nbIn;
                }
                ins = insHeap;
            }
            for (size_t k = 0; k < nbIn; k++) {
                OStream* s = &streams[sidx + k];
                size_t const inb = nbIn - 1 - k;
                if (!s->filled) FAIL(OZO_ERR_CORRUPTION);
                if ((int)inb < sg.nbSO) {
                    if (s->type != sg.soTypes[inb]) FAIL(OZO_ERR_CORRUPTION);
                } else if (!(s->type & sg.voType)) {
                    FAIL(OZO_ERR_CORRUPTION);
                }
                ins[inb] = s;
            }
            if (nodes[u].nbRegens != 1) FAIL(OZO_ERR_CORRUPTION);
            OStream* out = &streams[sidx + nbIn + nodes[u].dist[0]];
            if (out->filled) FAIL(OZO_ERR_CORRUPTION);
            int rc = dec_run(nodes[u].id, ins, nbIn, src + thStart + nodes[u].hdrStart,
                             nodes[u].hdrSize, out);
            if (rc) FAIL(-rc);
            /* a stream that references its input takes over the input's buffer */
            for (size_t k = 0; k < nbIn; k++) {
                OStream* s = &streams[sidx + k];
                if (s->own && out->p == s->p && !out->own) { out->own = s->own; s->own = NULL; }
                ost_free(s);
            }
            sidx += nbIn;
        }
        /* outputs: last nbOutputs slots, in reverse order */
        {
            /* content checksum: each output's bytes, and from v15 a string
             * output's lengths after its content (stream.c:727-773) */
            size_t catLen = 0;
            for (size_t o = 0; o < fh->nbOutputs; o++) {
                OStream* s = &streams[total - 1 - o];
                if (!s->filled) FAIL(OZO_ERR_CORRUPTION);
                catLen += s->n * s->w + (s->type == OZO_TYPE_STRING && ver >= 15 ? 4 * s->nbStrings : 0);
            }
            uint8_t* cat = (uint8_t*)malloc(catLen + 1);
            size_t cp = 0;
            for (size_t o = 0; o < fh->nbOutputs; o++) {
                OStream* s = &streams[total - 1 - o];
                size_t const b = s->n * s->w;
                memcpy(cat + cp, s->p, b);
                cp += b;
                if (s->type == OZO_TYPE_STRING) {
                    if (ver >= 15) {
                        for (size_t i = 0; i < s->nbStrings; i++) ozo_wr32(cat + cp + 4 * i, s->lens[i]);
                        cp += 4 * s->nbStrings;
                    }
                    outLens[o] = (uint32_t*)realloc(outLens[o], 4 * (outNbStrings[o] + s->nbStrings) + 4);
                    memcpy(outLens[o] + outNbStrings[o], s->lens, 4 * s->nbStrings);
                    outNbStrings[o] += s->nbStrings;
                }
                outBuf[o] = (uint8_t*)realloc(outBuf[o], outLen[o] + b + 1);
                memcpy(outBuf[o] + outLen[o], s->p, b);
                outLen[o] += b;
                if (outType[o] == 0) { outType[o] = s->type; outW[o] = s->w; }
                else if (outType[o] != s->type || outW[o] != s->w) { free(cat); FAIL(OZO_ERR_CORRUPTION); }
            }
            if (hasContentCk && (uint32_t)ozo_xxh3_64(cat, catLen) != contentCk) {
                free(cat);
                FAIL(OZO_ERR_CHECKSUM);
            }
            free(cat);
        }
        ret = (int64_t)(pos - start);
    }
done:
#undef FAIL
    if (streams) {
        size_t total = ns;
        for (size_t u = 0; u < nd; u++) total += nodes[u].nbRegens;
        for (size_t i = 0; i < total; i++) ost_free(&streams[i]);
    }
    free(streams);
    free(nodes);
    free(tmp);
    free(trt);
    free(storedSizes);
    free(dists);
    free(insHeap);
    return ret;
}

int64_t ozo_decompressed_size(const void* src, size_t srcSize)
{
    FrameHdr fh;
    int64_t r = parse_frame_header(&fh, (const uint8_t*)src, srcSize);
    if (r < 0) return r;
    if (fh.nbOutputs != 1) return -OZO_ERR_UNSUPPORTED;
    return (int64_t)fh.sizes[0];
}

int64_t ozo_decompress(const void* srcv, size_t size, void* dst, size_t dstCap, int* outType,
                       int* outEltWidth)
{
    const uint8_t* src = (const uint8_t*)srcv;
    FrameHdr fh;
    int64_t r = parse_frame_header(&fh, src, size);
    if (r < 0) return r;
    if (fh.nbOutputs != 1) return -OZO_ERR_UNSUPPORTED;
    size_t pos = (size_t)r;
    uint8_t* bufs[1] = { NULL };
    size_t lens[1] = { 0 };
    int types[1] = { 0 };
    size_t ws[1] = { 0 };
    uint32_t* slens[1] = { NULL };
    size_t nbs[1] = { 0 };
    for (;;) {
        /* versions before 21 hold exactly one block and no end marker
         * (decompress2.c:1689-1714) */
        if (fh.version >= 21) {
            if (pos >= size) { free(bufs[0]); return -OZO_ERR_SRC_SIZE; }
            if (src[pos] == 0) { pos++; break; }
        }
        int64_t b = decode_block(&fh, src, size, pos, bufs, lens, types, ws, slens, nbs);
        if (b < 0) { free(bufs[0]); free(slens[0]); return b; }
        pos += (size_t)b;
        if (fh.version < 21) break;
    }
    free(slens[0]);
    if (lens[0] != fh.sizes[0]) { free(bufs[0]); return -OZO_ERR_CORRUPTION; }
    if (lens[0] > dstCap) { free(bufs[0]); return -OZO_ERR_DST_SIZE; }
    if (lens[0]) memcpy(dst, bufs[0], lens[0]);
    free(bufs[0]);
    if (outType) *outType = types[0] ? types[0] : fh.types[0];
    if (outEltWidth) *outEltWidth = (int)(ws[0] ? ws[0] : 1);
    return (int64_t)lens[0];
}

/* Decodes a frame of any number of outputs (ZL_DCtx_decompressMultiTBuffer,
 * decompress2.c:1590-1760). outs[o] receives a malloc'ed buffer (release it
 * with ozo_free), lens/types/widths its size, type and element width.
 * Returns the number of outputs, or a negative error. */
int64_t ozo_decompress_multi(const void* srcv, size_t size, size_t maxOut, void** outs, size_t* lens, int* types,
                             int* widths, void** strLens, size_t* nbStrings)
{
    const uint8_t* src = (const uint8_t*)srcv;
    FrameHdr fh;
    int64_t r = parse_frame_header(&fh, src, size);
    if (r < 0) return r;
    if (fh.nbOutputs > maxOut) return -OZO_ERR_DST_SIZE;
    size_t const no = fh.nbOutputs;
    uint8_t* bufs[OZO_MAX_OUTPUTS] = { NULL };
    size_t ln[OZO_MAX_OUTPUTS] = { 0 }, ws[OZO_MAX_OUTPUTS] = { 0 }, nbs[OZO_MAX_OUTPUTS] = { 0 };
    int ts[OZO_MAX_OUTPUTS] = { 0 };
    uint32_t* sl[OZO_MAX_OUTPUTS] = { NULL };
    size_t pos = (size_t)r;
    int64_t ret = (int64_t)no;
    for (;;) {
        if (fh.version >= 21) {
            if (pos >= size) { ret = -OZO_ERR_SRC_SIZE; break; }
            if (src[pos] == 0) { pos++; break; }
        }
        int64_t b = decode_block(&fh, src, size, pos, bufs, ln, ts, ws, sl, nbs);
        if (b < 0) { ret = b; break; }
        pos += (size_t)b;
        if (fh.version < 21) break;
    }
    for (size_t o = 0; o < no && ret >= 0; o++) {
        if (ln[o] != fh.sizes[o]) ret = -OZO_ERR_CORRUPTION;
        if (fh.version >= 21 && fh.types[o] == OZO_TYPE_STRING && nbs[o] != fh.nbStrings[o]) ret = -OZO_ERR_CORRUPTION;
    }
    for (size_t o = 0; o < no; o++) {
        if (ret < 0) {
            free(bufs[o]);
            free(sl[o]);
            continue;
        }
        outs[o] = bufs[o] ? bufs[o] : malloc(1);
        lens[o] = ln[o];
        types[o] = ts[o] ? ts[o] : fh.types[o];
        widths[o] = (int)(ws[o] ? ws[o] : 1);
        strLens[o] = sl[o] ? (void*)sl[o] : malloc(4);
        nbStrings[o] = nbs[o];
    }
    return ret;
}

void ozo_free(void* p) { free(p); }

/* Test entry point: runs one decoder on caller streams (codec-level known
 * answers). Inputs are given in the decoder's own order. */
int64_t ozo_decode_transform(unsigned id, const uint8_t* hdr, size_t hsz, size_t nbIn, const int* types,
                             const size_t* widths, const size_t* counts, const uint8_t* const* data, void* out,
                             size_t outCap, int* outType, size_t* outW, size_t* outN)
{
    OStream ins[16];
    OStream* pin[16];
    if (nbIn > 16) return -OZO_ERR_UNSUPPORTED;
    for (size_t i = 0; i < nbIn; i++) {
        memset(&ins[i], 0, sizeof(ins[i]));
        ost_ref(&ins[i], types[i], widths[i], counts[i], data[i]);
        pin[i] = &ins[i];
    }
    OStream o;
    memset(&o, 0, sizeof(o));
    int rc = dec_run(id, pin, nbIn, hdr, hsz, &o);
    if (rc < 0) return rc;
    size_t const bytes = o.n * o.w;
    int64_t ret = (int64_t)bytes;
    if (bytes > outCap) ret = -OZO_ERR_DST_SIZE;
    else if (bytes) memcpy(out, o.p, bytes);
    if (outType) *outType = o.type;
    if (outW) *outW = o.w;
    if (outN) *outN = o.n;
    ost_free(&o);
    return ret;
}

