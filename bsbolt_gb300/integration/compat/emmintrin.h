/*
 * emmintrin.h -- the SSE2 subset that BWA's ksw.c uses, for hosts without SSE2.
 *
 * A GB300 node's host CPU is an Arm (Grace) core: BWA's striped Smith-Waterman
 * (ksw.c, `#include <emmintrin.h>` at ksw.c:29, the only SIMD file of the BWA
 * fork) does not build there.  Putting this directory first on the include
 * path (-I<repo>/bsbolt_gb300/integration/compat) lets the unmodified BWA
 * sources compile on such a host.  On AArch64 every operation is one or two
 * NEON instructions; elsewhere it is a scalar loop over the 16 bytes.
 *
 * Semantics follow the Intel intrinsics guide, lane i being byte/word i of the
 * little-endian 128-bit value:
 *   _mm_adds_epu8 / _mm_subs_epu8     unsigned saturating byte add / subtract
 *   _mm_max_epu8, _mm_cmpeq_epi8      unsigned byte max, byte equality (0xff / 0)
 *   _mm_adds_epi16, _mm_max_epi16     signed saturating word add, signed word max
 *   _mm_subs_epu16, _mm_cmpgt_epi16   unsigned saturating word subtract, signed word >
 *   _mm_movemask_epi8                 bit i = top bit of byte i
 *   _mm_extract_epi16(a, i)           word i, zero-extended
 *   _mm_slli_si128 / _mm_srli_si128   whole-register byte shifts toward higher / lower lanes
 * Only the operations ksw.c calls are provided.  Never included on x86-64 builds
 * unless asked for (the system header wins there without this -I).
 */
#ifndef BSB_COMPAT_EMMINTRIN_H
#define BSB_COMPAT_EMMINTRIN_H

#include <stdint.h>
#include <string.h>

/* 16 bytes, 16-byte aligned; may alias the int8_t/int16_t profile writes of ksw_qinit */
typedef long long __m128i __attribute__((__vector_size__(16), __aligned__(16), __may_alias__));

#define BSB_SSE_INLINE static inline __attribute__((__always_inline__, __unused__))

BSB_SSE_INLINE __m128i _mm_load_si128(const __m128i *p) { return *p; }
BSB_SSE_INLINE void _mm_store_si128(__m128i *p, __m128i a) { *p = a; }

#if defined(__aarch64__) && defined(__ARM_NEON)
#include <arm_neon.h>

#define BSB_U8(a) ((uint8x16_t)(a))
#define BSB_U16(a) ((uint16x8_t)(a))
#define BSB_S16(a) ((int16x8_t)(a))
#define BSB_M(a) ((__m128i)(a))

BSB_SSE_INLINE __m128i _mm_set1_epi8(char c) { return BSB_M(vdupq_n_u8((uint8_t)c)); }
BSB_SSE_INLINE __m128i _mm_set1_epi16(short w) { return BSB_M(vdupq_n_s16((int16_t)w)); }
BSB_SSE_INLINE __m128i _mm_set1_epi32(int d) { return BSB_M(vdupq_n_s32((int32_t)d)); }

BSB_SSE_INLINE __m128i _mm_adds_epu8(__m128i a, __m128i b) { return BSB_M(vqaddq_u8(BSB_U8(a), BSB_U8(b))); }
BSB_SSE_INLINE __m128i _mm_subs_epu8(__m128i a, __m128i b) { return BSB_M(vqsubq_u8(BSB_U8(a), BSB_U8(b))); }
BSB_SSE_INLINE __m128i _mm_max_epu8(__m128i a, __m128i b) { return BSB_M(vmaxq_u8(BSB_U8(a), BSB_U8(b))); }
BSB_SSE_INLINE __m128i _mm_cmpeq_epi8(__m128i a, __m128i b) { return BSB_M(vceqq_u8(BSB_U8(a), BSB_U8(b))); }
BSB_SSE_INLINE __m128i _mm_adds_epi16(__m128i a, __m128i b) { return BSB_M(vqaddq_s16(BSB_S16(a), BSB_S16(b))); }
BSB_SSE_INLINE __m128i _mm_max_epi16(__m128i a, __m128i b) { return BSB_M(vmaxq_s16(BSB_S16(a), BSB_S16(b))); }
BSB_SSE_INLINE __m128i _mm_subs_epu16(__m128i a, __m128i b) { return BSB_M(vqsubq_u16(BSB_U16(a), BSB_U16(b))); }
BSB_SSE_INLINE __m128i _mm_cmpgt_epi16(__m128i a, __m128i b) { return BSB_M(vcgtq_s16(BSB_S16(a), BSB_S16(b))); }

BSB_SSE_INLINE int _mm_movemask_epi8(__m128i a)
{
    /* top bit of each byte, weighted by 1 << (lane % 8), summed per half */
    static const uint8_t w[16] = {1, 2, 4, 8, 16, 32, 64, 128, 1, 2, 4, 8, 16, 32, 64, 128};
    const uint8x16_t bits = vandq_u8(vshrq_n_u8(BSB_U8(a), 7), vdupq_n_u8(1));
    const uint8x16_t m = vmulq_u8(bits, vld1q_u8(w));
    return (int)vaddv_u8(vget_low_u8(m)) | (int)vaddv_u8(vget_high_u8(m)) << 8;
}

#define _mm_extract_epi16(a, i) ((int)vgetq_lane_u16(BSB_U16(a), (i)))
/* byte shifts by an immediate 1..15: vext takes 16 - n bytes from one side and n from the other */
#define _mm_slli_si128(a, n) BSB_M(vextq_u8(vdupq_n_u8(0), BSB_U8(a), 16 - (n)))
#define _mm_srli_si128(a, n) BSB_M(vextq_u8(BSB_U8(a), vdupq_n_u8(0), (n)))

#else /* portable scalar form */

typedef union { __m128i v; uint8_t b[16]; uint16_t w[8]; int16_t s[8]; } bsb_m128_lanes;

BSB_SSE_INLINE __m128i _mm_set1_epi8(char c)
{
    bsb_m128_lanes r;
    memset(r.b, (uint8_t)c, 16);
    return r.v;
}
BSB_SSE_INLINE __m128i _mm_set1_epi16(short x)
{
    bsb_m128_lanes r;
    int i;
    for (i = 0; i < 8; ++i) r.s[i] = (int16_t)x;
    return r.v;
}
BSB_SSE_INLINE __m128i _mm_set1_epi32(int x)
{
    bsb_m128_lanes r;
    int i;
    for (i = 0; i < 4; ++i) memcpy(r.b + 4 * i, &x, 4);
    return r.v;
}

#define BSB_SSE_BYTEWISE(name, expr)                                       \
    BSB_SSE_INLINE __m128i name(__m128i a_, __m128i b_)                    \
    {                                                                      \
        bsb_m128_lanes a, b, r;                                            \
        int i;                                                             \
        a.v = a_, b.v = b_;                                                \
        for (i = 0; i < 16; ++i) {                                         \
            const int x = a.b[i], y = b.b[i];                              \
            r.b[i] = (uint8_t)(expr);                                      \
        }                                                                  \
        return r.v;                                                        \
    }
#define BSB_SSE_WORDWISE(name, expr)                                       \
    BSB_SSE_INLINE __m128i name(__m128i a_, __m128i b_)                    \
    {                                                                      \
        bsb_m128_lanes a, b, r;                                            \
        int i;                                                             \
        a.v = a_, b.v = b_;                                                \
        for (i = 0; i < 8; ++i) {                                          \
            const int sx = a.s[i], sy = b.s[i], ux = a.w[i], uy = b.w[i];  \
            (void)sx, (void)sy, (void)ux, (void)uy;                        \
            r.w[i] = (uint16_t)(expr);                                     \
        }                                                                  \
        return r.v;                                                        \
    }

BSB_SSE_BYTEWISE(_mm_adds_epu8, x + y > 255 ? 255 : x + y)
BSB_SSE_BYTEWISE(_mm_subs_epu8, x > y ? x - y : 0)
BSB_SSE_BYTEWISE(_mm_max_epu8, x > y ? x : y)
BSB_SSE_BYTEWISE(_mm_cmpeq_epi8, x == y ? 0xff : 0)
BSB_SSE_WORDWISE(_mm_adds_epi16, sx + sy > 32767 ? 32767 : sx + sy < -32768 ? -32768 : sx + sy)
BSB_SSE_WORDWISE(_mm_max_epi16, sx > sy ? sx : sy)
BSB_SSE_WORDWISE(_mm_subs_epu16, ux > uy ? ux - uy : 0)
BSB_SSE_WORDWISE(_mm_cmpgt_epi16, sx > sy ? 0xffff : 0)

BSB_SSE_INLINE int _mm_movemask_epi8(__m128i a_)
{
    bsb_m128_lanes a;
    int i, m = 0;
    a.v = a_;
    for (i = 0; i < 16; ++i) m |= (a.b[i] >> 7) << i;
    return m;
}
BSB_SSE_INLINE int bsb_sse_extract_epi16(__m128i a_, int i)
{
    bsb_m128_lanes a;
    a.v = a_;
    return a.w[i & 7];
}
BSB_SSE_INLINE __m128i bsb_sse_bslli(__m128i a_, int n)
{
    bsb_m128_lanes a, r;
    int i;
    a.v = a_;
    for (i = 0; i < 16; ++i) r.b[i] = i >= n ? a.b[i - n] : 0;
    return r.v;
}
BSB_SSE_INLINE __m128i bsb_sse_bsrli(__m128i a_, int n)
{
    bsb_m128_lanes a, r;
    int i;
    a.v = a_;
    for (i = 0; i < 16; ++i) r.b[i] = i + n < 16 ? a.b[i + n] : 0;
    return r.v;
}
#define _mm_extract_epi16(a, i) bsb_sse_extract_epi16((a), (i))
#define _mm_slli_si128(a, n) bsb_sse_bslli((a), (n))
#define _mm_srli_si128(a, n) bsb_sse_bsrli((a), (n))

#undef BSB_SSE_BYTEWISE
#undef BSB_SSE_WORDWISE
#endif

#endif /* BSB_COMPAT_EMMINTRIN_H */
