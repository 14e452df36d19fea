// ksw_core.cuh -- the warp-cooperative, bit-exact ksw_extend2 (ksw.c:380-479).
//
// Shared by the batched extension kernels (ksw_extend.cu) and the per-read
// chain extension (chain.cu).  See ksw_extend.cu for the design notes.
#pragma once

#include <climits>

#include "bsb_internal.cuh"

struct KswResult {
    int score, qle, tle, gtle, gscore, max_off;
    long long cells;
};

// Sign-extended byte of x chosen by a prmt selector (bit 3 of each selector
// nibble replicates the sign of the chosen byte, PTX ISA prmt.b32 default mode).
__device__ __forceinline__ int prmt_sext(uint32_t x, uint32_t sel)
{
    uint32_t r;
    asm("prmt.b32 %0, %1, 0, %2;" : "=r"(r) : "r"(x), "r"(sel));
    return (int)r;
}

// Scores of target bases 0..3 against query base qc, one per byte:
// mat[c*5 + qc] for c = 0..3.  The matrix is only indexed with constants
// (selecting on qc), which keeps the kernel parameters out of local memory.
__device__ __forceinline__ uint32_t profile_word(const KswParams &P, int qc)
{
    uint32_t w[5];
#pragma unroll
    for (int b = 0; b < 5; ++b)
        w[b] = (uint32_t)(uint8_t)P.mat[b] | (uint32_t)(uint8_t)P.mat[5 + b] << 8 |
               (uint32_t)(uint8_t)P.mat[10 + b] << 16 | (uint32_t)(uint8_t)P.mat[15 + b] << 24;
    return qc == 0 ? w[0] : qc == 1 ? w[1] : qc == 2 ? w[2] : qc == 3 ? w[3] : w[4];
}

// mat[20 + qc]: the score of an N in the target against query base qc.
__device__ __forceinline__ int profile_n(const KswParams &P, int qc)
{
    return qc == 0 ? P.mat[20] : qc == 1 ? P.mat[21] : qc == 2 ? P.mat[22] : qc == 3 ? P.mat[23] : P.mat[24];
}

__device__ __forceinline__ uint32_t sext_selector(int byte)
{
    const uint32_t b = (uint32_t)byte, r = b | 8u;
    return b | r << 4 | r << 8 | r << 12;
}

// Extends one job with the calling warp (every lane returns the same tuple).
// All control values are warp-uniform.  Acc supplies query base j and target
// base i (q(j), t(i)), so jobs can read a byte buffer or the 2-bit reference.
//
// Register state per lane, columns j = lane*C + s:
//   Hs[s] = eh[j].h = H(i-1, j-1),  Es[s] = eh[j].e = E(i, j)   (ksw.c:376-378)
// Invariant: every column left of the band (j < beg) holds H = E = 0.  The
// reference never reads those cells again (beg only grows), and with them at
// zero the F scan and the row maximum need no left-edge masks: a dead column
// has M = 0, T = 0, V = e_ins*(j+1), F = 0 and H = 0.  The shrink step only
// moves beg over cells that are already zero; when the band edge i-w moves
// beg instead, the cells it passes are zeroed explicitly.
template <int C, class Acc>
__device__ __forceinline__ KswResult ksw_warp(const KswParams &P, int qlen, int tlen, int h0, int w_in,
                                              int end_bonus, const Acc &acc, int lane)
{
    const int o_del = P.o_del, e_del = P.e_del, o_ins = P.o_ins, e_ins = P.e_ins;
    const int oe_del = o_del + e_del, oe_ins = o_ins + e_ins;
    const int base = lane * C;

    // query profile: byte c of prof[s] = mat[c*5 + q[j]] for target bases 0..3;
    // the N row (target base 4) is kept apart in profN, four slots per word.
    uint32_t prof[C];
    uint32_t profN[(C + 3) / 4];
    int Hs[C], Es[C];
#pragma unroll
    for (int s = 0; s < (C + 3) / 4; ++s) profN[s] = 0;
    const int h1run = max(h0 - oe_ins, 0);
#pragma unroll
    for (int s = 0; s < C; ++s) {
        const int j = base + s;
        const int qc = j < qlen ? acc.q(j) : 0;
        prof[s] = profile_word(P, qc);
        profN[s >> 2] |= (uint32_t)(uint8_t)profile_n(P, qc) << ((s & 3) * 8);
        // first row: h0, then an insertion run clipped at zero (ksw.c:395-397)
        Hs[s] = j == 0 ? h0 : (j <= qlen ? max(h1run - e_ins * (j - 1), 0) : 0);
        Es[s] = 0;
    }

    // band clamp (ksw.c:399-407)
    int w = w_in;
    {
        int max_ins = band_cap(qlen * P.mat_max + end_bonus - o_ins, e_ins);
        max_ins = max_ins > 1 ? max_ins : 1;
        w = w < max_ins ? w : max_ins;
        int max_del = band_cap(qlen * P.mat_max + end_bonus - o_del, e_del);
        max_del = max_del > 1 ? max_del : 1;
        w = w < max_del ? w : max_del;
    }

    int best = h0, best_i = -1, best_j = -1, max_ie = -1, gscore = -1, max_off = 0;
    int beg = 0, end = qlen;
    long long ncell = 0;
    const int q_lane = qlen / C, q_slot = qlen % C;   // owner of column qlen

    // target bases arrive 32 rows at a time, one byte per lane, next chunk prefetched
    uint32_t tch = lane < tlen ? (uint32_t)acc.t(lane) : 4u;
    uint32_t tnext = 32 + lane < tlen ? (uint32_t)acc.t(32 + lane) : 4u;

    for (int i = 0; i < tlen; ++i) {
        const int tc = (int)__shfl_sync(BSB_FULL_MASK, tch, i & 31);
        if ((i & 31) == 31) {
            tch = tnext;
            const int ti = i + 33 + lane;
            tnext = ti < tlen ? (uint32_t)acc.t(ti) : 4u;
        }
        // band of this row (ksw.c:416-419)
        if (beg < i - w) {
            beg = i - w;
#pragma unroll
            for (int s = 0; s < C; ++s)
                if (base + s < beg) Hs[s] = 0, Es[s] = 0;
        }
        if (end > i + w + 1) end = i + w + 1;
        if (end > qlen) end = qlen;
        // H(i,-1) (ksw.c:421-424)
        const int h1_init = beg == 0 ? max(h0 - (o_del + e_del * (i + 1)), 0) : 0;

        if (beg >= end) {
            // empty band: the reference's loop does not run, eh[end] gets {h1,0},
            // the query-end test sees j == beg, and the zero row max stops it.
            if (beg == qlen) {
                max_ie = gscore > h1_init ? max_ie : i;
                gscore = gscore > h1_init ? gscore : h1_init;
            }
            break;
        }

        // ---- pass 1: M, next-row E, and the F-scan operand V = T(j) + e_ins*(j+1)
        int Mv[C], En[C], Pf[C];
        int run = 0;
        if (tc < 4) {
            const uint32_t sel = sext_selector(tc);
#pragma unroll
            for (int s = 0; s < C; ++s) {
                const int j = base + s;
                const int sc = prmt_sext(prof[s], sel);
                const int Hp = Hs[s];
                const int M = Hp ? Hp + sc : 0;
                const int Ti = __viaddmax_s32(M, -oe_ins, 0);
                En[s] = __viaddmax_s32(Es[s], -e_del, __viaddmax_s32(M, -oe_del, 0));
                run = max(run, Ti + e_ins * (j + 1));
                Pf[s] = run;
                Mv[s] = M;
            }
        } else {
#pragma unroll
            for (int s = 0; s < C; ++s) {
                const int j = base + s;
                const int sc = prmt_sext(profN[s >> 2], sext_selector(s & 3));
                const int Hp = Hs[s];
                const int M = Hp ? Hp + sc : 0;
                const int Ti = __viaddmax_s32(M, -oe_ins, 0);
                En[s] = __viaddmax_s32(Es[s], -e_del, __viaddmax_s32(M, -oe_del, 0));
                run = max(run, Ti + e_ins * (j + 1));
                Pf[s] = run;
                Mv[s] = M;
            }
        }

        // ---- warp exclusive prefix max of the lane totals (lane 0 starts from 0 = F at column 0)
        int incl = run;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) incl = max(incl, __shfl_up_sync(BSB_FULL_MASK, incl, d));
        const int excl = __shfl_up_sync(BSB_FULL_MASK, incl, 1);
        const int carry = lane == 0 ? 0 : excl;

        // ---- pass 2: H, the row-max key (H << 10 | j), and the new eh[] (H shifted one column)
        int kmax = -1, prevH = 0;
        uint32_t nzb = 0;
#pragma unroll
        for (int s = 0; s < C; ++s) {
            const int j = base + s;
            const int G = s == 0 ? carry : max(carry, Pf[s - 1]);
            const int F = G - e_ins * j;
            const int H = __vimax3_s32(Mv[s], Es[s], F);
            const bool lt = j < end;
            if (lt) kmax = max(kmax, H * 1024 + j);     // ties keep the later column (ksw.c:437)
            const int nE = lt ? En[s] : 0;     // E beyond end is 0 at every row (ksw_group16.cuh, pass 2)
            Es[s] = nE;
            if (s > 0) {
                const int nH = j <= end ? prevH : Hs[s];
                Hs[s] = nH;
                if (j <= end && (nH | nE) != 0) nzb |= 1u << s;
            }
            prevH = H;
        }
        {
            int Hleft = __shfl_up_sync(BSB_FULL_MASK, prevH, 1);
            if (lane == 0) Hleft = h1_init;
            const int nH = base <= end ? Hleft : Hs[0];
            Hs[0] = nH;
            if (base <= end && (nH | Es[0]) != 0) nzb |= 1u;
        }

        ncell += end - beg;
        const int kw = __reduce_max_sync(BSB_FULL_MASK, kmax);
        const int m = kw >> 10, mj = kw & 1023;

        if (end == qlen) {          // reached the query end: eh[qlen].h == H(i,qlen-1) (ksw.c:450-453)
            int hsel = 0;
#pragma unroll
            for (int s = 0; s < C; ++s) hsel = s == q_slot ? Hs[s] : hsel;
            const int h1 = __shfl_sync(BSB_FULL_MASK, hsel, q_lane);
            max_ie = gscore > h1 ? max_ie : i;
            gscore = gscore > h1 ? gscore : h1;
        }
        if (m == 0) break;                             // ksw.c:454
        if (m > best) {
            best = m, best_i = i, best_j = mj;
            const int d = mj > i ? mj - i : i - mj;
            max_off = max_off > d ? max_off : d;
        } else if (P.zdrop > 0) {                      // ksw.c:458-464
            const int di = i - best_i, dj = mj - best_j;
            if (di > dj) {
                if (best - m - (di - dj) * e_del > P.zdrop) break;
            } else {
                if (best - m - (dj - di) * e_ins > P.zdrop) break;
            }
        }
        // shrink to the non-zero cells (ksw.c:466-469); columns left of beg are zero
        const int lfirst = nzb ? base + __ffs(nzb) - 1 : INT_MAX;
        const int llast = nzb ? base + 31 - __clz(nzb) : -1;
        const int fnz = __reduce_min_sync(BSB_FULL_MASK, lfirst);
        const int lnz = __reduce_max_sync(BSB_FULL_MASK, llast);
        if (fnz < end) {
            beg = fnz;
            end = lnz + 2 < qlen ? lnz + 2 : qlen;
        } else {
            const int jj = lnz == end ? end : end - 1;
            beg = end;
            end = jj + 2 < qlen ? jj + 2 : qlen;
        }
    }
    KswResult r;
    r.score = best; r.qle = best_j + 1; r.tle = best_i + 1;
    r.gtle = max_ie + 1; r.gscore = gscore; r.max_off = max_off;
    r.cells = ncell;
    return r;
}

