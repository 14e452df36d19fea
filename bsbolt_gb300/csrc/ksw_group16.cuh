// ksw_group16.cuh -- ksw_group.cuh's row step on 16-bit cells, two columns per register.
//
// Same groups, rows, band logic, reductions and results as ksw_group_run (and so
// as ksw_extend2, ksw.c:380-479); what changes is the cell arithmetic.  A lane owns
// C = 2*C2 query columns and holds column u in the low half and column u + C2 in
// the high half of register u, as signed 16-bit values, so every cell operation --
// M = H + score (or 0), E, F, H = max(M, E, F), the band-edge selects -- is one
// 16x2 instruction for two cells (__viaddmax_s16x2, __vimax3_s16x2, ...).  The two
// halves are two runs of the row's F recurrence, over columns [0, C2) and
// [C2, C); the high run's carry-in is max(carry - e_ins*C2, F at the low run's
// end), so the group scan is unchanged.  The row maximum and its last column
// (ties keep the later column, ksw.c:437) are one maximum per half over the key
// H*16 + u, combined with the high half winning ties.
//
// Bounds: every H is at most h0 + qlen * max(mat) <= kPack16MaxH = 2047 (E, F <= H),
// so H*16 + u stays below 2^15; every subtraction is by a penalty or a column count
// (the launcher checks the penalties); with max(mat) <= 15, min(H + score, H*16) is
// H + score when H > 0 and at most 0 when H == 0, the reference's M (ksw.c:431) in
// every use.  The scheduler sends any other job of the shape to the 32-bit kernel.
#pragma once

#include "ksw_group.cuh"

constexpr int kPack16MaxH = 2047;
constexpr int kPack16MaxScore = 15;

__device__ __forceinline__ uint32_t pk16(int lo, int hi)
{
    return __byte_perm((uint32_t)lo, (uint32_t)hi, 0x5410);     // low halves of lo and hi
}
__device__ __forceinline__ int lo16(uint32_t x) { return (int)(int16_t)(x & 0xffffu); }
__device__ __forceinline__ int hi16(uint32_t x) { return (int)x >> 16; }

// Two source words, one byte each, sign-extended into the two halves:
// low half = byte b of x, high half = byte c of y (prmt's sign-replicate mode).
__device__ __forceinline__ uint32_t prmt2(uint32_t x, uint32_t y, uint32_t sel)
{
    uint32_t r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(x), "r"(y), "r"(sel));
    return r;
}
__host__ __device__ __forceinline__ constexpr uint32_t sext2_selector(int b, int c)
{
    return (uint32_t)b | ((uint32_t)b | 8u) << 4 | (uint32_t)(4 + c) << 8 | ((uint32_t)(4 + c) | 8u) << 12;
}

// sext2_selector(b, b) for a base b in 0..3 as one multiply-add: b * 0x1111 + 0xC480.
__host__ __device__ __forceinline__ constexpr uint32_t sext2_same(uint32_t b) { return b * 0x1111u + 0xC480u; }
static_assert(sext2_same(0) == sext2_selector(0, 0) && sext2_same(1) == sext2_selector(1, 1) &&
              sext2_same(2) == sext2_selector(2, 2) && sext2_same(3) == sext2_selector(3, 3),
              "the selector of a base");

// 1 in a half where u < the half of t (t - u >= 1), else 0.
__device__ __forceinline__ uint32_t below16(uint32_t t, int u)
{
    return __viaddmin_s16x2_relu(t, pk16(-u, -u), 0x00010001u);
}


// Pass 2 of a row over the lane's C2 registers (see ksw_group16_run): F from each half's carry-in,
// H, E(i+1,j), the row-maximum keys, the new eh[] and the non-zero bits.  Sym: o_del == o_ins and
// e_del == e_ins, so E and F share their gap-open term max(M - oe, 0).
template <int C2, bool Sym>
__device__ __forceinline__ void ksw16_pass2(const uint32_t (&Mv)[C2], uint32_t (&Es)[C2], uint32_t (&Hs)[C2],
                                            uint32_t &F, uint32_t t_lt, uint32_t &ltm_prev, uint32_t &kmx,
                                            uint32_t &Hprev, uint32_t &nE0, uint32_t &lem0, uint32_t &nzw,
                                            uint32_t ne_del, uint32_t noe_del, uint32_t ne_ins, uint32_t noe_ins)
{
    uint32_t kprev = 0;
#pragma unroll
    for (int u = 0; u < C2; ++u) {
        const uint32_t M = Mv[u], Eo = Es[u];
        const uint32_t H = __vimax3_s16x2(M, Eo, F);
        const uint32_t td = __viaddmax_s16x2_relu(M, noe_del, 0);
        const uint32_t ti = Sym ? td : __viaddmax_s16x2_relu(M, noe_ins, 0);
        const uint32_t En = __viaddmax_s16x2(Eo, ne_del, td);
        F = __viaddmax_s16x2(F, ne_ins, ti);
        const uint32_t ltm = below16(t_lt, u) * 0xffffu, lem = ltm_prev;
        ltm_prev = ltm;
        const uint32_t key = (H & ltm) * 16u + pk16(u, u);             // ties: the later column
        if (u & 1) kmx = __vimax3_s16x2(kmx, kprev, key);              // two registers a step
        else kprev = key;
        const uint32_t nE = En & ltm;
        Es[u] = nE;
        if (u > 0) {
            const uint32_t nH = (Hprev & lem) | (Hs[u] & ~lem);
            Hs[u] = nH;
            // 1 in a half where nH or nE is non-zero (both >= 0, their sum < 2^15); the
            // halves' bits are distinct, so + is |: one shift-add
            nzw += __viaddmin_s16x2_relu(nH, nE, 0x00010001u) << u;
        } else {
            nE0 = nE, lem0 = lem;
        }
        Hprev = H;
    }
    if (C2 & 1) kmx = __vimax_s16x2_relu(kmx, kprev);
}

template <int C2, int G>
__device__ __forceinline__ void ksw_group16_run(const KswParams &P, const bsb_ext_job_t *__restrict__ jobs,
                                                const uint8_t *__restrict__ seq, const int32_t *__restrict__ order,
                                                int lo, int hi, int *__restrict__ counter,
                                                bsb_ext_out_t *__restrict__ out, int64_t *__restrict__ cells)
{
    static_assert(C2 <= 16, "the row-maximum key and the non-zero bits hold a column index in 4 bits per half");
    constexpr int C = 2 * C2;
    const int lane = threadIdx.x & 31, gl = lane & (G - 1);
    const unsigned gm = group_mask<G>(lane);
    const int e_del = P.e_del, e_ins = P.e_ins;
    const int oe_del = P.o_del + e_del, oe_ins = P.o_ins + e_ins;
    const int base = gl * C;
    const int eC = e_ins * C;
    const uint32_t ne_del = pk16(-e_del, -e_del), ne_ins = pk16(-e_ins, -e_ins);
    const uint32_t noe_del = pk16(-oe_del, -oe_del), noe_ins = pk16(-oe_ins, -oe_ins);
    const bool sym_gaps = oe_del == oe_ins && e_del == e_ins;

    // per-group job state
    int qlen = 0, tlen = 0, h0 = 0, w = 0, job = -1;
    const uint8_t *t = nullptr;
    uint32_t prof[C];
    uint32_t profN[(C + 3) / 4];
    uint32_t Hs[C2], Es[C2];
    int best = 0, best_i = -1, best_j = -1, max_ie = -1, gscore = -1, max_off = 0, beg = 0, end = 0, i = 0;
    long long ncell = 0;
    int q_lane = 0, q_slot = 0;
    uint32_t tch = 4u, tnext = 4u;
#pragma unroll
    for (int s = 0; s < C; ++s) prof[s] = 0;
#pragma unroll
    for (int u = 0; u < C2; ++u) Hs[u] = 0, Es[u] = 0;
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
                int h_init[C];
#pragma unroll
                for (int s = 0; s < C; ++s) {
                    const int j = base + s;
                    const int qc = j < qlen ? q[j] : 0;
                    prof[s] = profile_word(P, qc);
                    profN[s >> 2] |= (uint32_t)(uint8_t)profile_n(P, qc) << ((s & 3) * 8);
                    h_init[s] = j == 0 ? h0 : (j <= qlen ? max(h1run - e_ins * (j - 1), 0) : 0);   // ksw.c:395-397
                }
#pragma unroll
                for (int u = 0; u < C2; ++u) Hs[u] = pk16(h_init[u], h_init[u + C2]), Es[u] = 0;
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

        // ---- one target row of this group's job (ksw.c:412-470); per-job decisions
        // are selects or warp-uniform branches, as in ksw_group_run.
        const int tc = (int)__shfl_sync(act, tch, i & (G - 1), G);
        if ((i & (G - 1)) == G - 1) {
            tch = tnext;
            const int ti = i + G + 1 + gl;
            tnext = ti < tlen ? t[ti] : 4u;
        }
        const bool bump = beg < i - w;         // band edge (ksw.c:416-419)
        beg = bump ? i - w : beg;
        if (__any_sync(act, bump)) {           // cells left of the band are kept at zero
            // |beg - base| <= 1023 and u < C2: the 16-bit differences below are exact
            const uint32_t tb = pk16(beg - base, beg - base - C2);
#pragma unroll
            for (int u = 0; u < C2; ++u) {
                const uint32_t keep = ~(below16(tb, u) * 0xffffu);
                Hs[u] &= keep, Es[u] &= keep;
            }
        }
        end = min(end, i + w + 1);
        end = min(end, qlen);
        const int h1_init = beg == 0 ? max(h0 - (P.o_del + e_del * (i + 1)), 0) : 0;   // ksw.c:421-424
        const bool empty = beg >= end;         // empty band: the zero row max stops the job

        // pass 1: M, and the two halves' F runs from a zero carry-in (only their ends are
        // kept: pass 2 runs the recurrence again from the true carry-in, which keeps E(i+1, j)
        // and F out of the registers between the passes).
        // M = H(i-1,j-1) + score, or at most 0 when H(i-1,j-1) == 0 (ksw.c:431): the
        // minimum with H*16, which is >= H + score when H > 0 (scores <= 15).
        uint32_t Mv[C2];
        uint32_t local = 0;
        if (!__any_sync(act, tc >= 4)) {
            const uint32_t sel = sext2_same((uint32_t)tc);
#pragma unroll
            for (int u = 0; u < C2; ++u) {
                const uint32_t sc = prmt2(prof[u], prof[u + C2], sel);
                const uint32_t Hp = Hs[u];
                const uint32_t M = __viaddmin_s16x2(Hp, sc, Hp * 16u);   // Hp <= 2047: no carry between halves
                local = __viaddmax_s16x2(local, ne_ins, __viaddmax_s16x2_relu(M, noe_ins, 0));
                Mv[u] = M;
            }
        } else {                               // some group has an N in the target
            const uint32_t sel = sext2_same(tc < 4 ? (uint32_t)tc : 0u);
#pragma unroll
            for (int u = 0; u < C2; ++u) {
                const uint32_t sc = tc < 4 ? prmt2(prof[u], prof[u + C2], sel)
                                           : prmt2(profN[u >> 2], profN[(u + C2) >> 2],
                                                   sext2_selector(u & 3, (u + C2) & 3));
                const uint32_t Hp = Hs[u];
                const uint32_t M = __viaddmin_s16x2(Hp, sc, Hp * 16u);   // Hp <= 2047: no carry between halves
                local = __viaddmax_s16x2(local, ne_ins, __viaddmax_s16x2_relu(M, noe_ins, 0));
                Mv[u] = M;
            }
        }
        // the lane's map x -> max(x - e_ins*C, F_lane), then the group scan (ksw_group_run)
        const int f_lo_end = lo16(local);
        const int f_lane = max(f_lo_end - e_ins * C2, hi16(local));
        int incl = f_lane;
#pragma unroll
        for (int d = 1; d < G; d <<= 1)
            incl = __viaddmax_s32(__shfl_up_sync(act, incl, d, G), -eC * d, incl);
        const int excl = __shfl_up_sync(act, incl, 1, G);
        const int carry = gl == 0 ? 0 : excl;

        // pass 2: F (the recurrence F(i,j+1) = max(F(i,j) - e_ins, max(M - oe_ins, 0)) of
        // ksw.c:446-447 from each half's carry-in), H, E(i+1,j), the row maximum key, and the
        // new eh[] -- E(i+1, j) inside the band, 0 from end on; H shifted one column up to end,
        // kept beyond -- and the non-zero cells.  E beyond end is 0 in ksw_extend2 at every
        // row: eh[end].e is set to 0 (ksw.c:449), the columns the band shrinks off are those
        // past the last non-zero one (ksw.c:468), and the band's right edge moves at most
        // one column a row past them; so "kept beyond end" and "0" agree for E.  (H beyond
        // end can hold the first row's insertion run and is kept.)  Column 0's shifted H needs
        // the left lane's last column and column C2-1 of this lane, so it is finished after the loop.
        const int rend = end - base;               // |rend| <= 1023: exact in 16 bits
        // per half: ltm(u) = [column < rend]; lem(u) = [column <= rend] = ltm(u - 1)
        const uint32_t t_lt = pk16(rend, rend - C2);
        uint32_t ltm_prev = below16(t_lt, -1) * 0xffffu;
        uint32_t kmx = 0;                          // per half: max of H*16 + u over band columns
        uint32_t F = pk16(carry, max(carry - e_ins * C2, f_lo_end));   // F entering each half
        uint32_t Hprev = 0, nE0 = 0, lem0 = 0, nzw = 0;
        if (sym_gaps)                          // deletions and insertions cost alike: one gap-open term
            ksw16_pass2<C2, true>(Mv, Es, Hs, F, t_lt, ltm_prev, kmx, Hprev, nE0, lem0, nzw, ne_del, noe_del,
                                  ne_ins, noe_ins);
        else
            ksw16_pass2<C2, false>(Mv, Es, Hs, F, t_lt, ltm_prev, kmx, Hprev, nE0, lem0, nzw, ne_del, noe_del,
                                   ne_ins, noe_ins);
        int Hleft = __shfl_up_sync(act, hi16(Hprev), 1, G);
        if (gl == 0) Hleft = h1_init;
        {
            const uint32_t nH = (pk16(Hleft, lo16(Hprev)) & lem0) | (Hs[0] & ~lem0);
            Hs[0] = nH;
            nzw += __viaddmin_s16x2_relu(nH, nE0, 0x00010001u);
        }
        uint32_t nzb = (nzw & 0xffffu) | (nzw >> 16) << C2;
        nzb &= rend < 0 ? 0u : rend >= C - 1 ? 0xffffffffu : (2u << rend) - 1u;   // columns s <= rend
        // the lane's maximum: the high half (later columns) wins ties
        const int k_lo = lo16(kmx), k_hi = hi16(kmx);
        const int kmax = (k_hi >> 4) >= (k_lo >> 4) ? (k_hi >> 4) * 1024 + (k_hi & 15) + C2
                                                    : (k_lo >> 4) * 1024 + (k_lo & 15);
        const int kw = group_max<G>(act, kmax + base);
        const int m = kw >> 10, mj = kw & 1023;
        if (!empty) ncell += end - beg;

        // query end reached: eh[qlen].h == H(i, qlen-1), or h1 for an empty band at qlen (ksw.c:450-453)
        int hq = h1_init;
        if (__any_sync(act, !empty && end == qlen)) {
            // register qu by a select tree on its bits (C2 - 1 selects)
            const int qu = q_slot < C2 ? q_slot : q_slot - C2;
            uint32_t v[C2];
#pragma unroll
            for (int u = 0; u < C2; ++u) v[u] = Hs[u];
#pragma unroll
            for (int l = 0; (1 << l) < C2; ++l) {
                const bool b = (qu >> l) & 1;
#pragma unroll
                for (int a = 0; a + (1 << l) < C2; a += 2 << l) v[a] = b ? v[a + (1 << l)] : v[a];
            }
            const uint32_t wsel = v[0];
            const int hsel = q_slot < C2 ? lo16(wsel) : hi16(wsel);
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

        // shrink to the non-zero cells (ksw.c:466-469), as in ksw_group_run
        int fnz, lnz;
        if constexpr (G == 32) {
            fnz = __reduce_min_sync(act, nzb ? base + __ffs(nzb) - 1 : INT_MAX);
            lnz = __reduce_max_sync(act, nzb ? base + 31 - __clz(nzb) : -1);
        } else {
            const uint32_t pk = nzb ? (uint32_t)(2048 - base - __ffs(nzb)) << 16 | (uint32_t)(base + 32 - __clz(nzb)) : 0u;
            const uint32_t r = group_max_u16x2<G>(act, pk);
            fnz = 2047 - (int)(r >> 16);
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
