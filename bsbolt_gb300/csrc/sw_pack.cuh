// sw_pack.cuh -- ksw_align2's striped passes (bsbolt/External/BWA/ksw.c:111-327) with two
// SIMD lanes per thread, for sm_103a.
//
// The reference's results depend on its SSE2 striping (the query cut into slen segments of P
// lanes, column j + l*slen in lane l of segment j; F carried along a lane's stripe in the first
// pass, E and the row maximum taken from that pass, the lazy-F loop fixing H for the next row).
// Here thread t of a group of P/2 plays SIMD lanes t (low 16 bits) and t + P/2 (high 16 bits):
//   P = 16, byte lanes (ksw_u8): values 0..255 never leave 16 bits, so _mm_adds_epu8 is
//     min(a + b, 255) (__viaddmin_s16x2), _mm_subs_epu8 is max(a - b, 0) (__viaddmax_s16x2 of a
//     negated b), _mm_max_epu8 is __vimax_s16x2_relu (every value is non-negative);
//   P = 8, word lanes (ksw_i16): the same instructions with signed scores, for jobs whose scores
//     cannot reach the reference's 16-bit saturation (qlen * max score <= 32640) and whose
//     penalties stay below 32768, so that 16-bit arithmetic without saturation is exact.
// A job's H and E vectors and its query-profile selectors are register arrays sized by its
// segment count's bucket (below); the row's scores come from two profile words of its
// target base by one byte permute per pair of cells.  The lazy-F loop runs in closed form (see
// pack_pass).  The groups of a warp take consecutive jobs of a list sorted by segment count, so
// they run the same code for about as many rows.
#pragma once

#include <cstdint>

#include "bsb_internal.cuh"

namespace bsbsw {

constexpr int kXByte = 0x10000, kXStop = 0x20000, kXSubo = 0x40000, kXStart = 0x80000;
constexpr int kPackBlock = 128;
constexpr int kPackMaxSeg8 = 16;    // byte lanes: queries of up to 256 bases
constexpr int kPackMaxSeg16 = 40;   // word lanes: queries of up to 320 bases
// counter block of one lane width: [0..3] queues, [kRcnt + s] reverse passes of s segments,
// [kRcur + s] their scatter cursors
constexpr int kRcnt = 64, kRcur = 128, kCtrInts = 192;

struct PassOut {
    int score, te, qe, score2, te2;
};

struct PackParams {
    // per target base: the scores of query bases 0..3 (plo), of base 4, the padding column (score
    // 0) and zero (phi).  Byte lanes: biased, (uint8)(mat + shift); word lanes: signed bytes.
    uint32_t plo[5], phi[5];
    uint32_t nshift;                                       // byte lanes: -shift in both halves
    uint32_t npe_del, npoe_del, npe_ins, npoe_ins;         // negated penalties in both halves
    int shift, qmax, pe_ins;
};

// A pass's query and target: forward (qe = te = -1) or the reverse pass of ksw_align2
// (ksw.c:350): query[0..qe] reversed, target[0..te] reversed and the rest as is.
struct SwSeq {
    const uint8_t *q, *t;
    int qe, te;
    __device__ __forceinline__ int qc(int c) const { return qe < 0 ? q[c] : q[qe - c]; }
    __device__ __forceinline__ int tc(int i) const { return t[i <= te ? te - i : i]; }
};

__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel)   // bit 3 of a nibble: sign fill
{
    uint32_t d;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(sel));
    return d;
}

__host__ __device__ __forceinline__ uint32_t neg2(int v) { return (uint32_t)(uint16_t)(-v) * 0x10001u; }

template <int G>
__device__ __forceinline__ uint32_t lane_up(uint32_t x, int tid, unsigned gm)   // _mm_slli_si128 by one lane
{
    const uint32_t r = __shfl_sync(gm, x, (tid + G - 1) & (G - 1), G);
    return tid ? r : r << 16;
}

// maximum / minimum over the group's threads (G of them): a segmented butterfly, since a
// reduction with per-group member masks is carried out one mask at a time
template <int G>
__device__ __forceinline__ int grp_max(unsigned gm, int v)
{
#pragma unroll
    for (int d = G / 2; d > 0; d >>= 1) v = max(v, __shfl_xor_sync(gm, v, d, G));
    return v;
}

template <int G>
__device__ __forceinline__ int grp_min(unsigned gm, int v)
{
#pragma unroll
    for (int d = G / 2; d > 0; d >>= 1) v = min(v, __shfl_xor_sync(gm, v, d, G));
    return v;
}

// Segment counts per pass instance: a bucket of B consecutive counts (SLMAX - B, SLMAX] shares
// one instance, the exact count sl a runtime value: the striping uses sl, segments at and past
// sl are skipped (only the last B - 1 of the instance's segments test it).  Eight byte-lane and
// four word-lane instances keep the code the SMs run at one time small: with one instance per
// count, instruction fetch was the kernel's main stall.
template <int P>
constexpr int kSegBucket = P == 16 ? 2 : 8;

// One ksw_u8 (P = 16) or ksw_i16 (P = 8) pass of a group of P/2 threads on sl segments,
// SLMAX - kSegBucket < sl <= SLMAX.  hm: the thread's Hmax slots (stride kPackBlock); bbuf: the
// suboptimal rows (KSW_XSUBO only).
template <int P, int SLMAX>
__device__ __noinline__ PassOut pack_pass(const PackParams &S, const uint32_t *plo, const uint32_t *phi, int sl,
                                          int qlen, int tlen, const SwSeq &a, int xtra, uint32_t *hm, int2 *bbuf,
                                          int tid, unsigned gm)
{
    constexpr bool U8 = P == 16;
    constexpr int G = P / 2, SLMIN = SLMAX - kSegBucket<P> + 1;    // segments below SLMIN always exist
    const uint32_t nshift = S.nshift, npe_del = S.npe_del, npoe_del = S.npoe_del, npe_ins = S.npe_ins,
                   npoe_ins = S.npoe_ins;
    const int shift = S.shift, pe_ins = S.pe_ins;
    uint32_t sel[SLMAX], H[SLMAX], E[SLMAX];
#pragma unroll
    for (int j = 0; j < SLMAX; ++j) {              // ksw_qinit's striping; the vectors start at zero
        const int c0 = j + tid * sl, c1 = j + (tid + G) * sl;
        const bool in = j < sl;
        const uint32_t x = in && c0 < qlen ? (uint32_t)a.qc(c0) : 5u, y = in && c1 < qlen ? (uint32_t)a.qc(c1) : 5u;
        // bytes: score(x), 0 or its sign, score(y), 0 or its sign
        sel[j] = U8 ? (x | 0x60u | y << 8 | 0x6000u) : (x | (x | 8u) << 4 | y << 8 | (y | 8u) << 12);
        H[j] = 0, E[j] = 0;
        hm[j * kPackBlock] = 0;
    }
    const int minsc = (xtra & kXSubo) ? xtra & 0xffff : 0x10000;
    const int endsc = (xtra & kXStop) ? xtra & 0xffff : 0x10000;
    int gmax = 0, te = -1, n_b = 0, last_row = -2, last_sc = 0;
    int tc = tlen > 0 ? a.tc(0) : 0;
    uint32_t hlast = 0;                            // H of segment sl - 1 in the previous row
    for (int i = 0; i < tlen; ++i) {
        const int tn = i + 1 < tlen ? a.tc(i + 1) : 0;
        const uint32_t xlo = plo[tc], xhi = phi[tc];
        uint32_t h = lane_up<G>(hlast, tid, gm), f = 0, mx = 0;          // H(i-1, -1), ksw.c:141-142
        // H = max(a, E, f), a = the diagonal plus the score (ksw.c:149-153); the next f is
        // max(relu(f - e_ins), relu(H - oe_ins)) = max(relu(f - e_ins), relu(max(a, E) - oe_ins)), as
        // relu(f - oe_ins) <= relu(f - e_ins): one instruction per segment on the f chain
#pragma unroll
        for (int j = 0; j < SLMAX; ++j)
            if (j < SLMIN || j < sl) {
                const uint32_t s = prmt(xlo, xhi, sel[j]);
                const uint32_t ae = U8 ? __viaddmax_s16x2(__viaddmin_s16x2(h, s, 0x00ff00ffu), nshift, E[j])
                                       : __viaddmax_s16x2(h, s, E[j]);
                const uint32_t fo = __viaddmax_s16x2(ae, npoe_ins, 0u);
                const uint32_t hv = __vimax_s16x2_relu(ae, f);
                f = __viaddmax_s16x2(f, npe_ins, fo);
                mx = __vimax_s16x2_relu(mx, hv);
                E[j] = __viaddmax_s16x2(E[j], npe_del, __viaddmax_s16x2(hv, npoe_del, 0u));
                h = H[j];
                H[j] = hv;
            }
        {   // lazy F (ksw.c:166-177, 284-295).  The reference shifts f up one lane per round and
            // sweeps the segments until no lane can raise an H any more.  The sweep raises H(l, j)
            // to relu(G(l) - j*e_ins) at most, where G(l) is the F arriving at lane l's first
            // column: G(0) = 0, G(l) = max(x(l), relu(G(l-1) - sl*e_ins)), x(l) the f leaving lane
            // l-1; its early exit (Farrar's) leaves out only updates that change nothing.  So: the
            // reference's own first test, and where a lane fails it, G as a max-plus scan over the
            // lanes (the group's threads, then the low lanes into the high ones) and one max per
            // segment, without a vote per segment.  (Segments past sl take values nothing reads.)
            const uint32_t x = lane_up<G>(f, tid, gm);
            const uint32_t h0 = __vimax_s16x2_relu(H[0], x);
            const uint32_t hh = __viaddmax_s16x2(h0, npoe_ins, 0u), fn = __viaddmax_s16x2(x, npe_ins, 0u);
            if (__any_sync(gm, __vimax_s16x2_relu(fn, hh) != hh)) {
                const int d = pe_ins * sl;
                uint32_t g = x;
#pragma unroll
                for (int o = 1; o < G; o <<= 1) {
                    const uint32_t v = __shfl_up_sync(gm, g, o, G);
                    if (tid >= o) g = __viaddmax_s16x2(v, neg2(min(o * d, 32767)), g);
                }
                const int gl = (int)(__shfl_sync(gm, g, G - 1, G) & 0xffffu);
                g = __vimax_s16x2_relu(g, (uint32_t)max(gl - d * (tid + 1), 0) << 16);
#pragma unroll
                for (int j = 0; j < SLMAX; ++j) {
                    H[j] = __vimax_s16x2_relu(H[j], g);
                    g = __viaddmax_s16x2(g, npe_ins, 0u);
                }
            } else {
                H[0] = h0;
            }
        }
        hlast = H[SLMIN - 1];
#pragma unroll
        for (int j = SLMIN; j < SLMAX; ++j)
            if (j == sl - 1) hlast = H[j];
        const int imax = grp_max<G>(gm, max((int)(mx & 0xffffu), (int)(mx >> 16)));
        if (imax > gmax || imax >= minsc) {
            if (imax >= minsc) {                  // the rows of the suboptimal score (ksw.c:182-189)
                if (n_b == 0 || last_row + 1 != i) {
                    if (tid == 0) bbuf[n_b] = make_int2(imax, i);
                    ++n_b, last_row = i, last_sc = imax;
                } else if (last_sc < imax) {
                    if (tid == 0) bbuf[n_b - 1] = make_int2(imax, i);
                    last_row = i, last_sc = imax;
                }
            }
            if (imax > gmax) {
                gmax = imax, te = i;
#pragma unroll
                for (int j = 0; j < SLMAX; ++j) hm[j * kPackBlock] = H[j];
                if ((U8 && gmax + shift >= 255) || gmax >= endsc) break;
            }
        }
        tc = tn;
    }
    __syncwarp(gm);
    PassOut r;
    r.score = U8 ? (gmax + shift < 255 ? gmax : 255) : gmax;
    r.te = te, r.qe = -1, r.score2 = -1, r.te2 = -1;
    if (!U8 || r.score != 255) {
        int best = -1, col = 0x7fffffff;          // the smallest column holding the best Hmax value
#pragma unroll 1
        for (int j = 0; j < sl; ++j) {
            const uint32_t v = hm[j * kPackBlock];
            const int v0 = (int)(v & 0xffffu), v1 = (int)(v >> 16), c0 = j + tid * sl, c1 = j + (tid + G) * sl;
            if (v0 > best || (v0 == best && c0 < col)) best = v0, col = c0;
            if (v1 > best || (v1 == best && c1 < col)) best = v1, col = c1;
        }
        const int gbest = grp_max<G>(gm, best);
        r.qe = grp_min<G>(gm, best == gbest ? col : 0x7fffffff);
        if (n_b) {                                 // ksw.c:218-225: the best row outside te +- d
            const int d = (r.score + S.qmax - 1) / S.qmax, low = te - d, high = te + d;
            int bs = -1, bk = 0x7fffffff;
#pragma unroll 1
            for (int k = tid; k < n_b; k += G) {
                const int2 e = bbuf[k];
                if ((e.y < low || e.y > high) && e.x > bs) bs = e.x, bk = k;
            }
            const int gbs = grp_max<G>(gm, bs);
            const int gk = grp_min<G>(gm, bs == gbs ? bk : 0x7fffffff);
            if (gbs > r.score2 && gk != 0x7fffffff) r.score2 = gbs, r.te2 = bbuf[gk].y;
        }
    }
    return r;
}

// pack_pass of the bucket holding sl, for buckets ending at SLMAX..HI (step kSegBucket<P>).
// Each instance is a function of its own, so a kernel's registers are those of its largest.
template <int P, int SLMAX, int HI>
__device__ __forceinline__ PassOut pack_range(int sl, const PackParams &S, const uint32_t *plo, const uint32_t *phi,
                                              int qlen, int tlen, const SwSeq &a, int xtra, uint32_t *hm, int2 *bbuf,
                                              int tid, unsigned gm)
{
    if constexpr (SLMAX >= HI) {
        return pack_pass<P, HI>(S, plo, phi, sl, qlen, tlen, a, xtra, hm, bbuf, tid, gm);
    } else {
        if (sl <= SLMAX) return pack_pass<P, SLMAX>(S, plo, phi, sl, qlen, tlen, a, xtra, hm, bbuf, tid, gm);
        return pack_range<P, SLMAX + kSegBucket<P>, HI>(sl, S, plo, phi, qlen, tlen, a, xtra, hm, bbuf, tid, gm);
    }
}

// Jobs of LO..HI segments of P lanes (MAXS: the largest segment count of the lane width).
// REV = false: forward passes of list[0..n_fwd) (rsl[id] = the segment count of the reversed
// query when the job wants start positions, else 0; ctr[kRcnt + s] counts them).  REV = true:
// reverse passes of the jobs of list (grouped by segment count, the largest first, by
// sw_rev_scatter) whose reversed query has LO..HI segments, completing tb and qb.  Each warp
// takes 64/P consecutive jobs of its list at a time; q is the queue counter.
template <int P, bool REV, int LO, int HI, int MAXS>
__global__ void __launch_bounds__(kPackBlock, P == 16 ? 6 : 1)
sw_pack_kernel(PackParams S, const bsb_sw_job_t *__restrict__ jobs, const uint8_t *__restrict__ seq,
               const int32_t *__restrict__ list, int n_fwd, const int64_t *__restrict__ boff,
               int2 *__restrict__ bscratch, bsb_kswr_t *__restrict__ out, uint8_t *__restrict__ rsl,
               int *__restrict__ ctr, int *__restrict__ q)
{
    constexpr int G = P / 2, NG = 32 / G;
    __shared__ uint32_t hmax_s[HI * kPackBlock];
    __shared__ uint32_t plo[5], phi[5];
    if (threadIdx.x == 0) {
#pragma unroll
        for (int c = 0; c < 5; ++c) plo[c] = S.plo[c], phi[c] = S.phi[c];
    }
    __syncthreads();
    int total = n_fwd;
    if (REV) {                                   // this range's part of the reverse list
        int skip = 0;
        total = 0;
        for (int s = MAXS; s > HI; --s) skip += ctr[kRcnt + s];
        for (int s = HI; s >= LO; --s) total += ctr[kRcnt + s];
        list += skip;
    }
    const int wl = threadIdx.x & 31, g = wl / G, tid = wl % G;
    const unsigned gm = ((1u << G) - 1) << (G * g);
    uint32_t *hm = hmax_s + threadIdx.x;
    for (;;) {
        int base = 0;
        if (wl == 0) base = atomicAdd(q, NG);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= total) break;
        const int k = base + g;
        if (k < total) {
            const int id = list[k];
            const bsb_sw_job_t jb = jobs[id];
            const uint8_t *qp = seq + jb.qoff, *tp = seq + jb.toff;
            if (!REV) {
                const SwSeq a{qp, tp, -1, -1};
                constexpr int B0 = LO + kSegBucket<P> - 1;
                const PassOut r = pack_range<P, B0, HI>((jb.qlen + P - 1) / P, S, plo, phi, jb.qlen, jb.tlen, a,
                                                        jb.xtra, hm, bscratch + boff[id], tid, gm);
                const bool start = (jb.xtra & kXStart) && !((jb.xtra & kXSubo) && r.score < (jb.xtra & 0xffff));
                if (tid == 0) {
                    bsb_kswr_t o;
                    o.score = r.score, o.te = r.te, o.qe = r.qe, o.score2 = r.score2, o.te2 = r.te2;
                    o.tb = -1, o.qb = -1;
                    out[id] = o;
                    // a saturated byte pass leaves qe at -1, where the reference would profile no columns
                    const int sl = start && r.qe >= 0 ? (r.qe + P) / P : 0;
                    rsl[id] = (uint8_t)sl;
                    if (sl) atomicAdd(&ctr[kRcnt + sl], 1);
                }
            } else {
                const bsb_kswr_t o = out[id];
                const SwSeq a{qp, tp, o.qe, o.te};
                constexpr int B0 = LO + kSegBucket<P> - 1;
                const PassOut rr = pack_range<P, B0, HI>((o.qe + P) / P, S, plo, phi, o.qe + 1, jb.tlen, a,
                                                         kXStop | o.score, hm, nullptr, tid, gm);
                if (tid == 0 && rr.score == o.score) out[id].tb = o.te - rr.te, out[id].qb = o.qe - rr.qe;
            }
        }
        __syncwarp();
    }
}

// Lists the jobs of list[0..n) that want a reverse pass, grouped by its segment count (the
// largest first).
template <int MAXS>
__global__ void sw_rev_scatter(const int32_t *__restrict__ list, int n, const uint8_t *__restrict__ rsl,
                               int *__restrict__ ctr, int32_t *__restrict__ rlist)
{
    __shared__ int off[MAXS + 1];
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int s = MAXS; s >= 1; --s) off[s] = acc, acc += ctr[kRcnt + s];
    }
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int id = list[i], s = rsl[id];
        if (s) rlist[off[s] + atomicAdd(&ctr[kRcur + s], 1)] = id;
    }
}

// One sw_pack_kernel launch on st: the forward passes of list[0..n) or (rev) the reverse passes
// of this range.  ctr: the lane width's counter block; ctr[q] the queue.
template <int P, int LO, int HI, int MAXS>
cudaError_t sw_pack_run(bool rev, const PackParams &S, const bsb_sw_job_t *jobs, const uint8_t *seq,
                        const int32_t *list, int n, const int64_t *boff, int2 *bscratch, bsb_kswr_t *out,
                        uint8_t *rsl, int *ctr, int q, int n_sm, cudaStream_t st)
{
    static int resident[2] = {};
    if (!resident[0]) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident[0], sw_pack_kernel<P, false, LO, HI, MAXS>,
                                                      kPackBlock, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident[1], sw_pack_kernel<P, true, LO, HI, MAXS>,
                                                      kPackBlock, 0);
        resident[0] = resident[0] > 0 ? resident[0] : 1, resident[1] = resident[1] > 0 ? resident[1] : 1;
    }
    const int per_block = kPackBlock * 2 / P;              // jobs in flight per block
    const int64_t want = ((int64_t)n + per_block - 1) / per_block, cap = (int64_t)n_sm * resident[rev ? 1 : 0];
    const int grid = (int)(want < cap ? want : cap);
    if (grid <= 0) return cudaSuccess;
    if (rev)
        sw_pack_kernel<P, true, LO, HI, MAXS><<<grid, kPackBlock, 0, st>>>(S, jobs, seq, list, 0, boff, bscratch,
                                                                           out, rsl, ctr, ctr + q);
    else
        sw_pack_kernel<P, false, LO, HI, MAXS><<<grid, kPackBlock, 0, st>>>(S, jobs, seq, list, n, boff, bscratch,
                                                                            out, rsl, ctr, ctr + q);
    return cudaGetLastError();
}

// The word-lane ranges, each in a translation unit of its own (sw_pack16a.cu: 1..16 segments,
// sw_pack16b.cu: 17..40) so that they compile side by side.
cudaError_t sw_pack16_run_lo(bool rev, const PackParams &S, const bsb_sw_job_t *jobs, const uint8_t *seq,
                             const int32_t *list, int n, const int64_t *boff, int2 *bscratch, bsb_kswr_t *out,
                             uint8_t *rsl, int *ctr, int q, int n_sm, cudaStream_t st);
cudaError_t sw_pack16_run_hi(bool rev, const PackParams &S, const bsb_sw_job_t *jobs, const uint8_t *seq,
                             const int32_t *list, int n, const int64_t *boff, int2 *bscratch, bsb_kswr_t *out,
                             uint8_t *rsl, int *ctr, int q, int n_sm, cudaStream_t st);

}  // namespace bsbsw
