/* Shared helpers of the CPU oracle (test infrastructure only). */
#ifndef OZO_INTERNAL_H
#define OZO_INTERNAL_H

#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "ozl_oracle.h"

#define OZO_TYPE_SERIAL 1
#define OZO_TYPE_STRUCT 2
#define OZO_TYPE_NUMERIC 4
#define OZO_TYPE_STRING 8

/* Standard transform IDs of the wire format (src/openzl/common/wire_format.h:211-306). */
enum {
    TR_DELTA_INT = 1,
    TR_ZIGZAG = 3,
    TR_TRANSPOSE_SPLIT = 4,
    TR_CONV_SERIAL_TO_STRUCT = 5,
    TR_CONV_STRUCT_TO_SERIAL = 6,
    TR_CONV_STRUCT_TO_NUM_LE = 7,
    TR_CONV_NUM_TO_STRUCT_LE = 8,
    TR_CONV_SERIAL_TO_NUM_LE = 9,
    TR_CONV_NUM_TO_SERIAL_LE = 10,
    TR_SEPARATE_STRING = 12, /* content + lengths -> string */
    TR_BITPACK_SERIAL = 27,
    TR_BITPACK_INT = 28,
    TR_FLATPACK = 29,
    TR_FLOAT_DECONSTRUCT = 33,
    TR_TOKENIZE_FIXED = 36,
    TR_TOKENIZE_NUMERIC = 37,
    TR_SPLITN = 40,
    TR_CONSTANT_SERIAL = 44,
    TR_CONSTANT_FIXED = 45,
    TR_SPLITN_STRUCT = 47,
    TR_SPLITN_NUM = 48,
    TR_FSE_V2 = 49,
    TR_HUFFMAN_V2 = 50,
    TR_HUFFMAN_STRUCT_V2 = 51,
    TR_FSE_NCOUNT = 52,
    TR_END = 63,
};

#define OZO_MAGIC_BASE 0xD7B1A5C0u

/* Little-endian loads (the oracle runs on little-endian hosts; the
 * byte-swap keeps it correct elsewhere). */
static inline uint64_t ozo_le(uint64_t v, size_t n)
{
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_BIG_ENDIAN__
    v = __builtin_bswap64(v) >> (64 - 8 * n);
#else
    (void)n;
#endif
    return v;
}
static inline uint16_t ozo_rd16(const uint8_t* p) { return (uint16_t)(p[0] | (p[1] << 8)); }
static inline uint32_t ozo_rd32(const uint8_t* p)
{
    uint32_t v;
    memcpy(&v, p, 4);
    return (uint32_t)ozo_le(v, 4);
}
static inline uint64_t ozo_rd64(const uint8_t* p)
{
    uint64_t v;
    memcpy(&v, p, 8);
    return ozo_le(v, 8);
}
static inline uint64_t ozo_rdN(const uint8_t* p, size_t n)
{
    switch (n) {
        case 1: return p[0];
        case 2: return ozo_rd16(p);
        case 4: return ozo_rd32(p);
        case 8: return ozo_rd64(p);
        default: {
            uint64_t v = 0;
            for (size_t i = 0; i < n; i++) v |= (uint64_t)p[i] << (8 * i);
            return v;
        }
    }
}
static inline void ozo_wr16(uint8_t* p, uint16_t v) { p[0] = (uint8_t)v; p[1] = (uint8_t)(v >> 8); }
static inline void ozo_wr32(uint8_t* p, uint32_t v)
{
    v = (uint32_t)ozo_le(v, 4);
    memcpy(p, &v, 4);
}
static inline void ozo_wr64(uint8_t* p, uint64_t v)
{
    v = ozo_le(v, 8);
    memcpy(p, &v, 8);
}
static inline int ozo_highbit32(uint32_t v) { return 31 - __builtin_clz(v); }
static inline int ozo_highbit64(uint64_t v) { return 63 - __builtin_clzll(v); }
/* Smallest n with (1 << n) >= v (src/openzl/shared/bits.h:227). */
static inline int ozo_nextpow2(uint64_t v)
{
    int n = 0;
    while (n < 64 && ((uint64_t)1 << n) < v) n++;
    return n;
}

/* LEB128 varint (src/openzl/shared/varint.h). Returns 0 on success. */
static inline int ozo_varint_dec(const uint8_t** pp, const uint8_t* end, uint64_t* out)
{
    const uint8_t* p = *pp;
    uint64_t v = 0;
    for (int shift = 0; shift < 70; shift += 7) {
        if (p >= end) return -1;
        uint8_t b = *p++;
        v |= (uint64_t)(b & 0x7f) << shift;
        if (!(b & 0x80)) { *pp = p; *out = v; return 0; }
    }
    return -1;
}
static inline size_t ozo_varint_enc(uint8_t* dst, uint64_t v)
{
    size_t n = 0;
    while (v >= 0x80) { dst[n++] = (uint8_t)(v | 0x80); v >>= 7; }
    dst[n++] = (uint8_t)v;
    return n;
}

#endif
