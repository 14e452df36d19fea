// fm_index.cuh -- device view of the FM-index and the occurrence primitives.
//
// The occurrence array holds the reference's information (bwt.h:70-78,
// bwtindex.c:151-173: per 128 BWT symbols four uint64 cumulative counts and
// eight uint32 words of 2-bit symbols) re-cut at upload into 32-byte sectors of
// 32 or 64 symbols that carry their own counts, so an occurrence query touches
// one 32-byte sector and counts inside two or four words instead of a 64-byte
// block and up to eight words.  Nothing else of the index is touched by a query.
#pragma once

#include <stdint.h>

struct DevFM {
    const uint4 *blk;        // 32-byte occurrence sectors (layouts below)
    const uint64_t *sb;      // 64-symbol layout: A, C, G counts before each 2^32-row superblock
    int sym64;               // 1: 64-symbol sectors, 0: 32-symbol sectors
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

// Device layouts of the occurrence array, built from the reference's at upload
// (occ_sectors_kernel / occ_sectors64_kernel, bsb_index.cu); either way an occurrence
// query reads one 32-byte sector (two 16-byte loads of one transaction) and T follows
// from the row:
//  - 32 symbols per sector (1 byte per symbol): the uint64 counts of A, C and G in the
//    rows before the sector's first symbol, then its two uint32 words of 2-bit symbols,
//    most significant pair first; a query counts inside at most two words.
//  - 64 symbols per sector (0.5 byte per symbol, the reference's density): the uint32
//    counts of A, C and G before the sector relative to its 2^32-row superblock (whose
//    uint64 counts sit in a small array, sb), one unused word, then four symbol words; a
//    query counts inside at most four words.  Half the bytes of the first layout, so an
//    index that would outgrow L2 keeps more of itself there.
constexpr int kSectorSyms = 32;

// Counts of A, C, G among the first n (0..16) symbols of x.
__device__ __forceinline__ void word_counts(uint32_t x, int n, uint32_t &a, uint32_t &c, uint32_t &g)
{
    const uint32_t keep = n >= 16 ? 0xffffffffu : ~(0xffffffffu >> (2 * n));
    const uint32_t hi = (x >> 1) & 0x55555555u, lo = x & 0x55555555u;
    a += __popc(~(hi | lo) & 0x55555555u & keep);
    c += __popc(lo & ~hi & keep);
    g += __popc(hi & ~lo & keep);
}

// Occurrences of each base in rows [0, kk] of the $-free BWT (bwt_occ4, bwt.c:169-187);
// kk is k after the $ adjustment.  *word receives the symbol word holding kk.
__device__ __forceinline__ Occ4 occ_at64(const DevFM &F, uint64_t kk, uint32_t *word)
{
    const uint4 *p = F.blk + (kk >> 6) * 2;
    const uint4 v0 = __ldg(p), v1 = __ldg(p + 1);
    const int n = (int)(kk & 63) + 1;                  // symbols counted in this sector
    uint32_t a = 0, c = 0, g = 0;
    word_counts(v1.x, n >= 16 ? 16 : n, a, c, g);
    word_counts(v1.y, n >= 32 ? 16 : n > 16 ? n - 16 : 0, a, c, g);
    word_counts(v1.z, n >= 48 ? 16 : n > 32 ? n - 32 : 0, a, c, g);
    word_counts(v1.w, n > 48 ? n - 48 : 0, a, c, g);
    uint64_t ba = 0, bc = 0, bg = 0;
    if (kk >> 32) {                                    // past the first 2^32 rows
        const uint64_t *b = F.sb + 3 * (kk >> 32);
        ba = __ldg(b), bc = __ldg(b + 1), bg = __ldg(b + 2);
    }
    Occ4 o;
    o.c[0] = ba + v0.x + a;
    o.c[1] = bc + v0.y + c;
    o.c[2] = bg + v0.z + g;
    o.c[3] = kk + 1 - o.c[0] - o.c[1] - o.c[2];
    if (word) {
        const int wi = (int)(kk & 63) >> 4;
        *word = wi == 0 ? v1.x : wi == 1 ? v1.y : wi == 2 ? v1.z : v1.w;
    }
    return o;
}

__device__ __forceinline__ Occ4 occ_at(const DevFM &F, uint64_t kk, uint32_t *word = nullptr)
{
    if (F.sym64) return occ_at64(F, kk, word);
    const uint4 *p = F.blk + (kk >> 5) * 2;
    const uint4 v0 = __ldg(p), v1 = __ldg(p + 1);
    const int pos = (int)(kk & 31);
    uint32_t a = 0, c = 0, g = 0;
    word_counts(v1.z, pos >= 16 ? 16 : pos + 1, a, c, g);
    word_counts(v1.w, pos >= 16 ? pos - 15 : 0, a, c, g);
    Occ4 o;
    o.c[0] = ((uint64_t)v0.y << 32 | v0.x) + a;
    o.c[1] = ((uint64_t)v0.w << 32 | v0.z) + c;
    o.c[2] = ((uint64_t)v1.y << 32 | v1.x) + g;
    o.c[3] = kk + 1 - o.c[0] - o.c[1] - o.c[2];
    if (word) *word = pos >= 16 ? v1.w : v1.z;
    return o;
}

__device__ __forceinline__ Occ4 occ4(const DevFM &F, uint64_t k)
{
    if (k == (uint64_t)-1) {
        Occ4 z;
        z.c[0] = z.c[1] = z.c[2] = z.c[3] = 0;
        return z;
    }
    return occ_at(F, k - (k >= F.primary));
}

// bwt_2occ4 (bwt.c:189-220) without branches, so the threads of a warp never split over
// whether k and l share a block.
__device__ __forceinline__ void occ4_pair(const DevFM &F, uint64_t k, uint64_t l, Occ4 &ok, Occ4 &ol)
{
    const bool kz = k == (uint64_t)-1, lz = l == (uint64_t)-1;
    const uint64_t kk = kz ? 0 : k - (k >= F.primary), ll = lz ? 0 : l - (l >= F.primary);
    ok = occ_at(F, kk);
    ol = occ_at(F, ll);
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

// One LF step of bwt_sa (bwt_invPsi, bwt.c:53-59): the row of the suffix one text
// position earlier; the primary row steps to row 0 (BWA's "$" convention).
__device__ __forceinline__ uint64_t lf_step(const DevFM &F, uint64_t k)
{
    if (k == F.primary) return 0;
    // the symbol row (bwt_invPsi uses k > primary, bwt.c:55) equals kk here, so one word serves both
    const uint64_t kk = k - (k >= F.primary);
    uint32_t x;
    const Occ4 o = occ_at(F, kk, &x);
    const int c = (int)(x >> ((~kk & 15) << 1) & 3);
    return l2_at(F, c) + (c == 0 ? o.c[0] : c == 1 ? o.c[1] : c == 2 ? o.c[2] : o.c[3]);
}
