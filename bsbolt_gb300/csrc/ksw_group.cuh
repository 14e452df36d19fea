// ksw_group.cuh -- batched ksw_extend2 with several jobs per warp.
//
// The same bit-exact row step as ksw_core.cuh (see the design notes there and
// in ksw_extend.cu), but a warp holds 32/G independent jobs, one per group of
// G lanes (G = 4, 8, 16 or 32), each lane owning C query columns.  What a row
// costs besides its cells -- the F prefix scan, the row-maximum and shrink
// reductions, the band and z-drop bookkeeping -- is executed once per warp
// for all its jobs, so it is amortised over up to eight jobs instead of one.
// Every group keeps its own row counter and fetches its next job as soon as
// the current one ends, so groups never wait for one another; a warp leaves
// only when the queue is empty and all its groups are done.
//
// The job state is kept in plain local variables (no aggregate), which keeps
// it in registers.
#pragma once

#include "ksw_core.cuh"

template <int G>
__device__ __forceinline__ unsigned group_mask(int lane)
{
    if (G == 32) return 0xffffffffu;
    return ((1u << G) - 1) << (lane & ~(G - 1));
}

// Maximum over the G lanes of each group.  A full warp uses the hardware
// reduction; smaller groups use a segmented butterfly, since a reduction with
// per-group member masks is carried out one mask at a time.
template <int G>
__device__ __forceinline__ int group_max(unsigned act, int v)
{
    if constexpr (G == 32) {
        return __reduce_max_sync(act, v);
    } else {
#pragma unroll
        for (int d = G / 2; d > 0; d >>= 1) v = max(v, __shfl_xor_sync(act, v, d, G));
        return v;
    }
}

// Per-halfword maximum over the G lanes of each group (values 0..32767).
template <int G>
__device__ __forceinline__ uint32_t group_max_u16x2(unsigned act, uint32_t v)
{
#pragma unroll
    for (int d = G / 2; d > 0; d >>= 1) v = __vimax_s16x2_relu(v, __shfl_xor_sync(act, v, d, G));
    return v;
}

// Persistent per-bin kernel body.  order[lo, hi) lists the bin's jobs in issue
// order; counter is the bin's queue head.
template <int C, int G>
__device__ __forceinline__ void ksw_group_run(const KswParams &P, const bsb_ext_job_t *__restrict__ jobs,
                                              const uint8_t *__restrict__ seq, const int32_t *__restrict__ order,
                                              int lo, int hi, int *__restrict__ counter,
                                              bsb_ext_out_t *__restrict__ out, int64_t *__restrict__ cells)
{
    static_assert(C <= 32, "the non-zero columns of a lane are a 32-bit mask");
    const int lane = threadIdx.x & 31, gl = lane & (G - 1);
    const unsigned gm = group_mask<G>(lane);
    const int e_del = P.e_del, e_ins = P.e_ins;
    const int oe_del = P.o_del + e_del, oe_ins = P.o_ins + e_ins;
    const int base = gl * C;
    const int eC = e_ins * C;

    // per-group job state
    int qlen = 0, tlen = 0, h0 = 0, w = 0, job = -1;
    const uint8_t *t = nullptr;
    uint32_t prof[C];
    uint32_t profN[(C + 3) / 4];
    int Hs[C], Es[C];
    int best = 0, best_i = -1, best_j = -1, max_ie = -1, gscore = -1, max_off = 0, beg = 0, end = 0, i = 0;
    long long ncell = 0;
    int q_lane = 0, q_slot = 0;
    uint32_t tch = 4u, tnext = 4u;
#pragma unroll
    for (int s = 0; s < C; ++s) prof[s] = 0, Hs[s] = 0, Es[s] = 0;
#pragma unroll
    for (int s = 0; s < (C + 3) / 4; ++s) profN[s] = 0;
    bool have = false, exhausted = false;

    for (;;) {
        if (!have && !exhausted) {            // this group takes its next job
            int idx = 0;
            if (gl == 0) idx = atomicAdd(counter, 1);
            idx = __shfl_sync(gm, idx, 0, G) + lo;
            if (idx < hi) {
                job = order[idx];
                const bsb_ext_job_t jb = jobs[job];
                qlen = jb.qlen; tlen = jb.tlen; h0 = jb.h0;
                const uint8_t *q = seq + jb.qoff;
                t = seq + jb.toff;
                const int h1run = max(h0 - oe_ins, 0);
#pragma unroll
                for (int s = 0; s < (C + 3) / 4; ++s) profN[s] = 0;
#pragma unroll
                for (int s = 0; s < C; ++s) {
                    const int j = base + s;
                    const int qc = j < qlen ? q[j] : 0;
                    prof[s] = profile_word(P, qc);
                    profN[s >> 2] |= (uint32_t)(uint8_t)profile_n(P, qc) << ((s & 3) * 8);
                    Hs[s] = j == 0 ? h0 : (j <= qlen ? max(h1run - e_ins * (j - 1), 0) : 0);   // ksw.c:395-397
                    Es[s] = 0;
                }
                w = jb.w;                                                                  // ksw.c:399-407
                {
                    int max_ins = band_cap(qlen * P.mat_max + jb.end_bonus - P.o_ins, e_ins);
                    max_ins = max_ins > 1 ? max_ins : 1;
                    w = w < max_ins ? w : max_ins;
                    int max_del = band_cap(qlen * P.mat_max + jb.end_bonus - P.o_del, e_del);
                    max_del = max_del > 1 ? max_del : 1;
                    w = w < max_del ? w : max_del;
                }
                best = h0; best_i = best_j = -1; max_ie = -1; gscore = -1; max_off = 0;
                beg = 0; end = qlen; i = 0; ncell = 0;
                q_lane = qlen / C; q_slot = qlen % C;
                tch = gl < tlen ? t[gl] : 4u;
                tnext = G + gl < tlen ? t[G + gl] : 4u;
                have = tlen > 0;
                if (!have && gl == 0) {        // no target: the reference returns h0 untouched
                    bsb_ext_out_t o;
                    o.score = h0; o.qle = 0; o.tle = 0; o.gtle = 0; o.gscore = -1; o.max_off = 0;
                    out[job] = o;
                    if (cells) cells[job] = 0;
                }
            } else {
                exhausted = true;
            }
        }
        const unsigned act = __ballot_sync(0xffffffffu, have);
        if (!act) break;
        if (!have) continue;

        // ---- one target row of this group's job (ksw.c:412-470).  Groups of a
        // warp sit at different rows of different jobs, so every per-job decision
        // below is a select, or a branch taken by the whole warp when any group
        // needs it (__any_sync) with the work predicated per group.
        const int tc = (int)__shfl_sync(act, tch, i & (G - 1), G);
        if ((i & (G - 1)) == G - 1) {
            tch = tnext;
            const int ti = i + G + 1 + gl;
            tnext = ti < tlen ? t[ti] : 4u;
        }
        const bool bump = beg < i - w;         // band edge (ksw.c:416-419)
        beg = bump ? i - w : beg;
        if (__any_sync(act, bump)) {           // cells left of the band are kept at zero
#pragma unroll
            for (int s = 0; s < C; ++s)
                if (base + s < beg) Hs[s] = 0, Es[s] = 0;
        }
        end = min(end, i + w + 1);
        end = min(end, qlen);
        const int h1_init = beg == 0 ? max(h0 - (P.o_del + e_del * (i + 1)), 0) : 0;   // ksw.c:421-424
        const bool empty = beg >= end;         // empty band: the zero row max stops the job

        // pass 1: M, next-row E, and F from a zero carry-in, F(j+1) = max(F(j) - e_ins, T(j)).
        // M = H(i-1,j-1) + score, or 0 when H(i-1,j-1) == 0 (ksw.c:431); min(Hp + sc, Hp << 8)
        // is that value whenever Hp > 0 and at most 0 when Hp == 0, which every use of M
        // (a maximum with a non-negative E, F or 0) cannot tell apart from 0.
        int Mv[C], En[C], Pf[C];
        int local = 0;
        if (!__any_sync(act, tc >= 4)) {
            const uint32_t sel = sext_selector(tc);
#pragma unroll
            for (int s = 0; s < C; ++s) {
                const int sc = prmt_sext(prof[s], sel);
                const int Hp = Hs[s];
                const int M = __viaddmin_s32(Hp, sc, Hp << 8);
                En[s] = __viaddmax_s32(Es[s], -e_del, __viaddmax_s32(M, -oe_del, 0));
                Pf[s] = local;
                local = __viaddmax_s32(local, -e_ins, __viaddmax_s32(M, -oe_ins, 0));
                Mv[s] = M;
            }
        } else {                               // some group has an N in the target
            const uint32_t sel = sext_selector(tc < 4 ? tc : 0);
#pragma unroll
            for (int s = 0; s < C; ++s) {
                const int sc = tc < 4 ? prmt_sext(prof[s], sel) : prmt_sext(profN[s >> 2], sext_selector(s & 3));
                const int Hp = Hs[s];
                const int M = __viaddmin_s32(Hp, sc, Hp << 8);
                En[s] = __viaddmax_s32(Es[s], -e_del, __viaddmax_s32(M, -oe_del, 0));
                Pf[s] = local;
                local = __viaddmax_s32(local, -e_ins, __viaddmax_s32(M, -oe_ins, 0));
                Mv[s] = M;
            }
        }
        // group scan of the lane maps x -> max(x - e_ins*C, local): F at each lane's first column
        int incl = local;
#pragma unroll
        for (int d = 1; d < G; d <<= 1)
            incl = __viaddmax_s32(__shfl_up_sync(act, incl, d, G), -eC * d, incl);
        const int excl = __shfl_up_sync(act, incl, 1, G);
        const int carry = gl == 0 ? 0 : excl;

        // pass 2: H, the row-max key (H << 10 | j), and the new eh[] (H shifted one column)
        // (columns are tested lane-relative, s against end - base)
        const int rend = end - base;
        int kmax = -1, prevH = 0;
        uint32_t nzb = 0;
#pragma unroll
        for (int s = 0; s < C; ++s) {
            const int F = __viaddmax_s32(carry, -e_ins * s, Pf[s]);
            const int H = __vimax3_s32(Mv[s], Es[s], F);
            const bool lt = s < rend;
            if (lt) kmax = max(kmax, H * 1024 + s);     // ties keep the later column (ksw.c:437)
            const int nE = lt ? En[s] : 0;     // E beyond end is 0 at every row (ksw_group16.cuh, pass 2)
            Es[s] = nE;
            if (s > 0) {
                const int nH = s <= rend ? prevH : Hs[s];
                Hs[s] = nH;
                if (s <= rend && (nH | nE) != 0) nzb |= 1u << s;
            }
            prevH = H;
        }
        {
            int Hleft = __shfl_up_sync(act, prevH, 1, G);
            if (gl == 0) Hleft = h1_init;
            const int nH = rend >= 0 ? Hleft : Hs[0];
            Hs[0] = nH;
            if (rend >= 0 && (nH | Es[0]) != 0) nzb |= 1u;
        }
        // A lane without a band column offers base - 1 < 1024: it can only win a row
        // whose maximum is 0, which ends the job before the column is used.
        const int kw = group_max<G>(act, kmax + base);
        const int m = kw >> 10, mj = kw & 1023;
        if (!empty) ncell += end - beg;

        // query end reached: eh[qlen].h == H(i, qlen-1), or h1 for an empty band at qlen (ksw.c:450-453)
        int hq = h1_init;
        if (__any_sync(act, !empty && end == qlen)) {
            int hsel = 0;
#pragma unroll
            for (int s = 0; s < C; ++s) hsel = s == q_slot ? Hs[s] : hsel;
            const int h1 = __shfl_sync(act, hsel, q_lane, G);
            hq = empty ? hq : h1;
        }
        if (empty ? beg == qlen : end == qlen) {
            max_ie = gscore > hq ? max_ie : i;
            gscore = gscore > hq ? gscore : hq;
        }

        // row maximum, z-drop (ksw.c:454-464)
        const bool live = !empty && m != 0;
        const bool up = live && m > best;
        const int di = i - best_i, dj = mj - best_j;
        const int drop = di > dj ? best - m - (di - dj) * e_del : best - m - (dj - di) * e_ins;
        const bool zd = live && !up && P.zdrop > 0 && drop > P.zdrop;
        if (up) {
            best = m, best_i = i, best_j = mj;
            const int d = mj > i ? mj - i : i - mj;
            max_off = max_off > d ? max_off : d;
        }

        // shrink to the non-zero cells (ksw.c:466-469)
        // first and last non-zero column, reduced together as (2047 - first, last + 1)
        int fnz, lnz;
        if constexpr (G == 32) {
            fnz = __reduce_min_sync(act, nzb ? base + __ffs(nzb) - 1 : INT_MAX);
            lnz = __reduce_max_sync(act, nzb ? base + 31 - __clz(nzb) : -1);
        } else {
            const uint32_t pk = nzb ? (uint32_t)(2048 - base - __ffs(nzb)) << 16 | (uint32_t)(base + 32 - __clz(nzb)) : 0u;
            const uint32_t r = group_max_u16x2<G>(act, pk);
            fnz = 2047 - (int)(r >> 16);       // 2047 (beyond any end) when the row has none
            lnz = (int)(r & 0xffffu) - 1;
        }
        const int jj = fnz < end ? lnz : (lnz == end ? end : end - 1);
        beg = fnz < end ? fnz : end;
        end = jj + 2 < qlen ? jj + 2 : qlen;
        ++i;
        const bool done = !live || zd || i >= tlen;
        if (done) {
            if (gl == 0) {
                bsb_ext_out_t o;
                o.score = best; o.qle = best_j + 1; o.tle = best_i + 1;
                o.gtle = max_ie + 1; o.gscore = gscore; o.max_off = max_off;
                out[job] = o;
                if (cells) cells[job] = ncell;
            }
            have = false;
        }
    }
}
