/* XXH3-64 (seed 0, default 192-byte secret), restated from the published
 * XXH3 algorithm. OpenZL uses its low 32 bits for the content and compressed
 * checksums (src/openzl/common/stream.c:727, src/openzl/decompress/
 * decompress2.c:1492-1570) and its low 8 bits for the frame-header checksum
 * (src/openzl/decompress/decode_frameheader.c:319). The secret and primes are
 * the algorithm's published constants. Test infrastructure only. */
#include "ozo_internal.h"

static const uint8_t kSecret[192] = {
    0xb8, 0xfe, 0x6c, 0x39, 0x23, 0xa4, 0x4b, 0xbe, 0x7c, 0x01, 0x81, 0x2c, 0xf7, 0x21, 0xad, 0x1c,
    0xde, 0xd4, 0x6d, 0xe9, 0x83, 0x90, 0x97, 0xdb, 0x72, 0x40, 0xa4, 0xa4, 0xb7, 0xb3, 0x67, 0x1f,
    0xcb, 0x79, 0xe6, 0x4e, 0xcc, 0xc0, 0xe5, 0x78, 0x82, 0x5a, 0xd0, 0x7d, 0xcc, 0xff, 0x72, 0x21,
    0xb8, 0x08, 0x46, 0x74, 0xf7, 0x43, 0x24, 0x8e, 0xe0, 0x35, 0x90, 0xe6, 0x81, 0x3a, 0x26, 0x4c,
    0x3c, 0x28, 0x52, 0xbb, 0x91, 0xc3, 0x00, 0xcb, 0x88, 0xd0, 0x65, 0x8b, 0x1b, 0x53, 0x2e, 0xa3,
    0x71, 0x64, 0x48, 0x97, 0xa2, 0x0d, 0xf9, 0x4e, 0x38, 0x19, 0xef, 0x46, 0xa9, 0xde, 0xac, 0xd8,
    0xa8, 0xfa, 0x76, 0x3f, 0xe3, 0x9c, 0x34, 0x3f, 0xf9, 0xdc, 0xbb, 0xc7, 0xc7, 0x0b, 0x4f, 0x1d,
    0x8a, 0x51, 0xe0, 0x4b, 0xcd, 0xb4, 0x59, 0x31, 0xc8, 0x9f, 0x7e, 0xc9, 0xd9, 0x78, 0x73, 0x64,
    0xea, 0xc5, 0xac, 0x83, 0x34, 0xd3, 0xeb, 0xc3, 0xc5, 0x81, 0xa0, 0xff, 0xfa, 0x13, 0x63, 0xeb,
    0x17, 0x0d, 0xdd, 0x51, 0xb7, 0xf0, 0xda, 0x49, 0xd3, 0x16, 0x55, 0x26, 0x29, 0xd4, 0x68, 0x9e,
    0x2b, 0x16, 0xbe, 0x58, 0x7d, 0x47, 0xa1, 0xfc, 0x8f, 0xf8, 0xb8, 0xd1, 0x7a, 0xd0, 0x31, 0xce,
    0x45, 0xcb, 0x3a, 0x8f, 0x95, 0x16, 0x04, 0x28, 0xaf, 0xd7, 0xfb, 0xca, 0xbb, 0x4b, 0x40, 0x7e,
};

#define P32_1 0x9E3779B1u
#define P32_2 0x85EBCA77u
#define P32_3 0xC2B2AE3Du
#define P64_1 0x9E3779B185EBCA87ull
#define P64_2 0xC2B2AE3D27D4EB4Full
#define P64_3 0x165667B19E3779F9ull
#define P64_4 0x85EBCA77C2B2AE63ull
#define P64_5 0x27D4EB2F165667C5ull
#define PMX1 0x165667919E3779F9ull
#define PMX2 0x9FB21C651E98DF25ull

static uint64_t fold128(uint64_t a, uint64_t b)
{
    unsigned __int128 p = (unsigned __int128)a * b;
    return (uint64_t)p ^ (uint64_t)(p >> 64);
}
static uint64_t rotl64(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }
static uint64_t avalanche(uint64_t h)
{
    h ^= h >> 37;
    h *= PMX1;
    return h ^ (h >> 32);
}
static uint64_t xxh64_avalanche(uint64_t h)
{
    h ^= h >> 33;
    h *= P64_2;
    h ^= h >> 29;
    h *= P64_3;
    return h ^ (h >> 32);
}
static uint64_t mix16(const uint8_t* in, const uint8_t* sec)
{
    return fold128(ozo_rd64(in) ^ ozo_rd64(sec), ozo_rd64(in + 8) ^ ozo_rd64(sec + 8));
}
/* lane i gains the neighbouring lane's input word and the product of its
 * own keyed word's halves; the stripe is loaded first and each lane updated
 * once, so the compiler can vectorize the eight lanes */
static inline void accumulate512(uint64_t acc[8], const uint8_t* in, const uint8_t* sec)
{
    uint64_t v[8], k[8];
    for (int i = 0; i < 8; i++) {
        v[i] = ozo_rd64(in + 8 * i);
        k[i] = v[i] ^ ozo_rd64(sec + 8 * i);
    }
    for (int i = 0; i < 8; i++) acc[i] += v[i ^ 1] + (uint64_t)(uint32_t)k[i] * (k[i] >> 32);
}
static void scramble(uint64_t acc[8], const uint8_t* sec)
{
    for (int i = 0; i < 8; i++) {
        uint64_t a = acc[i];
        a ^= a >> 47;
        a ^= ozo_rd64(sec + 8 * i);
        acc[i] = a * P32_1;
    }
}

uint64_t ozo_xxh3_64(const void* src, size_t len)
{
    const uint8_t* in = (const uint8_t*)src;
    const uint8_t* s = kSecret;
    if (len <= 16) {
        if (len > 8) {
            uint64_t lo = ozo_rd64(in) ^ (ozo_rd64(s + 24) ^ ozo_rd64(s + 32));
            uint64_t hi = ozo_rd64(in + len - 8) ^ (ozo_rd64(s + 40) ^ ozo_rd64(s + 48));
            uint64_t acc = (uint64_t)len + __builtin_bswap64(lo) + hi + fold128(lo, hi);
            return avalanche(acc);
        }
        if (len >= 4) {
            uint64_t i1 = ozo_rd32(in), i2 = ozo_rd32(in + len - 4);
            uint64_t k = (i2 + (i1 << 32)) ^ (ozo_rd64(s + 8) ^ ozo_rd64(s + 16));
            k ^= rotl64(k, 49) ^ rotl64(k, 24);
            k *= PMX2;
            k ^= (k >> 35) + len;
            k *= PMX2;
            return k ^ (k >> 28);
        }
        if (len > 0) {
            uint32_t c = ((uint32_t)in[0] << 16) | ((uint32_t)in[len >> 1] << 24) | in[len - 1]
                    | ((uint32_t)len << 8);
            uint64_t k = (uint64_t)c ^ (uint64_t)(ozo_rd32(s) ^ ozo_rd32(s + 4));
            return xxh64_avalanche(k);
        }
        return xxh64_avalanche(ozo_rd64(s + 56) ^ ozo_rd64(s + 64));
    }
    if (len <= 128) {
        uint64_t acc = len * P64_1;
        if (len > 32) {
            if (len > 64) {
                if (len > 96) {
                    acc += mix16(in + 48, s + 96);
                    acc += mix16(in + len - 64, s + 112);
                }
                acc += mix16(in + 32, s + 64);
                acc += mix16(in + len - 48, s + 80);
            }
            acc += mix16(in + 16, s + 32);
            acc += mix16(in + len - 32, s + 48);
        }
        acc += mix16(in, s);
        acc += mix16(in + len - 16, s + 16);
        return avalanche(acc);
    }
    if (len <= 240) {
        uint64_t acc = len * P64_1;
        size_t rounds = len / 16;
        for (size_t i = 0; i < 8; i++) acc += mix16(in + 16 * i, s + 16 * i);
        acc = avalanche(acc);
        for (size_t i = 8; i < rounds; i++) acc += mix16(in + 16 * i, s + 16 * (i - 8) + 3);
        acc += mix16(in + len - 16, s + 136 - 17);
        return avalanche(acc);
    }
    uint64_t acc[8] = { P32_3, P64_1, P64_2, P64_3, P64_4, P32_2, P64_5, P32_1 };
    size_t const blockLen = 1024;
    size_t const nbBlocks = (len - 1) / blockLen;
    for (size_t b = 0; b < nbBlocks; b++) {
        for (size_t st = 0; st < 16; st++) accumulate512(acc, in + b * blockLen + 64 * st, s + 8 * st);
        scramble(acc, s + 192 - 64);
    }
    size_t const nbStripes = ((len - 1) - blockLen * nbBlocks) / 64;
    for (size_t st = 0; st < nbStripes; st++) accumulate512(acc, in + nbBlocks * blockLen + 64 * st, s + 8 * st);
    accumulate512(acc, in + len - 64, s + 192 - 64 - 7);
    uint64_t r = len * P64_1;
    for (int i = 0; i < 4; i++)
        r += fold128(acc[2 * i] ^ ozo_rd64(s + 11 + 16 * i), acc[2 * i + 1] ^ ozo_rd64(s + 11 + 16 * i + 8));
    return avalanche(r);
}
