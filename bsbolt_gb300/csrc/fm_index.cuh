// fm_index.cuh -- device view of the FM-index and the occurrence primitives.
//
// Layout in HBM is the reference's own (bwt.h:70-78, bwtindex.c:151-173):
// one 64-byte block per 128 BWT symbols -- four uint64 cumulative counts,
// then eight uint32 words of 2-bit symbols, most significant pair first.
// A block is fetched as four 16-byte vector loads (one 64 B, two-sector
// transaction); nothing else of the index is touched by an occurrence query.
#pragma once

#include <stdint.h>

struct DevFM {
    const uint4 *blk;        // 64-byte occurrence blocks
    const uint64_t *sa;      // sampled suffix array, sa[0] = (uint64_t)-1
    const uint64_t *sa_full; // every row's bwt_sa value (seq_len + 1 entries), or NULL
    uint64_t primary;
    uint64_t seq_len;
    uint64_t L2[5];
    int sa_shift;            // log2(sa_intv)
};

struct DevIntv {             // bwtintv_t (bwt.h:60-62)
    uint64_t x0, x1, x2, info;
};

struct Occ4 {
    uint64_t c[4];
};

// 64-byte block holding (already $-adjusted) BWT position k.
struct Block {
    uint4 w[4];
};

// One LF step of bwt_sa (bwt_invPsi, bwt.c:53-59): the row of the suffix one text
// position earlier; the primary row steps to row 0 (BWA's "$" convention).
__device__ __forceinline__ uint64_t lf_step(const DevFM &F, uint64_t k);

__device__ __forceinline__ Block load_block(const DevFM &F, uint64_t kk)
{
    const uint4 *p = F.blk + ((kk >> 7) << 2);
    Block b;
    b.w[0] = __ldg(p + 0);
    b.w[1] = __ldg(p + 1);
    b.w[2] = __ldg(p + 2);
    b.w[3] = __ldg(p + 3);
    return b;
}

__device__ __forceinline__ uint32_t block_word(const Block &b, int i)
{
    const uint4 &v = b.w[2 + (i >> 2)];
    switch (i & 3) {
    case 0: return v.x;
    case 1: return v.y;
    case 2: return v.z;
    default: return v.w;
    }
}

// Counts of A, C, G (T follows from the total) among the first n symbols of x.
__device__ __forceinline__ void word_counts(uint32_t x, int n, uint32_t &a, uint32_t &c, uint32_t &g)
{
    const uint32_t keep = n >= 16 ? 0xffffffffu : ~(0xffffffffu >> (2 * n));
    const uint32_t hi = (x >> 1) & 0x55555555u, lo = x & 0x55555555u;
    a += __popc(~(hi | lo) & 0x55555555u & keep);
    c += __popc(lo & ~hi & keep);
    g += __popc(hi & ~lo & keep);
}

// Occurrences of each base in rows [0, k] of the $-free BWT, from a loaded block
// (bwt_occ4, bwt.c:169-187).  kk is k after the $ adjustment.
__device__ __forceinline__ Occ4 occ_in_block(const Block &b, uint64_t kk)
{
    const int pos = (int)(kk & 127);
    const int last = pos >> 4;
    uint32_t a = 0, c = 0, g = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int n = i < last ? 16 : (i == last ? (pos & 15) + 1 : 0);
        if (n) word_counts(block_word(b, i), n, a, c, g);
    }
    const uint32_t t = (uint32_t)pos + 1 - a - c - g;
    Occ4 o;
    o.c[0] = (((uint64_t)b.w[0].y) << 32 | b.w[0].x) + a;
    o.c[1] = (((uint64_t)b.w[0].w) << 32 | b.w[0].z) + c;
    o.c[2] = (((uint64_t)b.w[1].y) << 32 | b.w[1].x) + g;
    o.c[3] = (((uint64_t)b.w[1].w) << 32 | b.w[1].z) + t;
    return o;
}

__device__ __forceinline__ Occ4 occ4(const DevFM &F, uint64_t k)
{
    if (k == (uint64_t)-1) {
        Occ4 z;
        z.c[0] = z.c[1] = z.c[2] = z.c[3] = 0;
        return z;
    }
    const uint64_t kk = k - (k >= F.primary);
    return occ_in_block(load_block(F, kk), kk);
}

// bwt_2occ4 (bwt.c:189-220) without branches: both blocks are always loaded (the same
// 64 bytes twice when k and l share a 128-symbol bucket, the second from L1), so the
// threads of a warp never split over which case they are in.
__device__ __forceinline__ void occ4_pair(const DevFM &F, uint64_t k, uint64_t l, Occ4 &ok, Occ4 &ol)
{
    const bool kz = k == (uint64_t)-1, lz = l == (uint64_t)-1;
    const uint64_t kk = kz ? 0 : k - (k >= F.primary), ll = lz ? 0 : l - (l >= F.primary);
    const Block bk = load_block(F, kk), bl = load_block(F, ll);
    ok = occ_in_block(bk, kk);
    ol = occ_in_block(bl, ll);
    if (kz) ok.c[0] = ok.c[1] = ok.c[2] = ok.c[3] = 0;
    if (lz) ol.c[0] = ol.c[1] = ol.c[2] = ol.c[3] = 0;
}

// F.L2[i] for i = 0..4, indexed with constants only (a dynamic index would copy the
// kernel parameter to local memory).
__device__ __forceinline__ uint64_t l2_at(const DevFM &F, int i)
{
    return i == 0 ? F.L2[0] : i == 1 ? F.L2[1] : i == 2 ? F.L2[2] : i == 3 ? F.L2[3] : F.L2[4];
}

__device__ __forceinline__ DevIntv set_intv(const DevFM &F, int c)   // bwt.h:80
{
    DevIntv r;
    r.x0 = l2_at(F, c) + 1;
    r.x2 = l2_at(F, c + 1) - l2_at(F, c);
    r.x1 = l2_at(F, 3 - c) + 1;
    r.info = 0;
    return r;
}

__device__ __forceinline__ uint64_t lf_step(const DevFM &F, uint64_t k)
{
    if (k == F.primary) return 0;
    const uint64_t kk = k - (k >= F.primary);
    const Block b = load_block(F, kk);
    const uint64_t xs = k - (k > F.primary);        // symbol row (bwt_invPsi uses >, bwt.c:55)
    const int c = (int)(block_word(b, (int)((xs & 127) >> 4)) >> ((~xs & 15) << 1) & 3);
    // xs and kk differ only when k == primary, handled above, so one block serves both
    const Occ4 o = occ_in_block(b, kk);
    return l2_at(F, c) + (c == 0 ? o.c[0] : c == 1 ? o.c[1] : c == 2 ? o.c[2] : o.c[3]);
}
