// sw.cu -- ksw_align2 (bsbolt/External/BWA/ksw.c:336-360), the local Smith-Waterman of mate
// rescue (mem_matesw, bwamem_pair.c:111-180), for batches of jobs on sm_103a.
//
// The reference is SSE2 striped code whose results depend on the striping: the query is
// cut into slen segments of P lanes (P = 16 one-byte lanes with KSW_XBYTE, else 8 two-byte
// lanes), column j + l*slen in lane l of segment j; each target row is one pass over the
// segments (F runs within a lane's stripe only, and E is taken from that pass's H) and then
// a lazy-F loop that carries F across stripes, one lane shift per round, until no lane can
// still raise an H; the row maximum comes from the first pass and covers the padded columns
// past the query end.  So each job runs on a group of P GPU lanes, lane l playing SIMD lane
// l, with the reference's saturating 8- or 16-bit arithmetic, its lane shifts (__shfl_up_sync)
// and its all-lanes exit tests (__any_sync over the group).  The group's H0/H1/E/Hmax vectors
// live in its slice of shared memory, segment-major like the reference's.
//
//   sw_pack_kernel<16, ..> byte-lane jobs of 1..16 segments (every mate of < 250 bases with
//                          BWA's scoring), two SIMD lanes per thread (sw_pack.cuh): forward
//                          passes in the order of a host counting sort by segments and length,
//                          sw_rev_scatter grouping the jobs that want start positions by the
//                          segment count of their reversed query, then their reverse passes
//   sw_pack_kernel<8, ..>  the same for word-lane jobs of 1..40 segments whose scores stay
//                          clear of 16-bit saturation (sw_pack16a.cu, sw_pack16b.cu), on a
//                          second stream
//   sw_kernel<16>, <8>     every other job (longer queries, extreme scores or penalties, empty
//                          queries): one SIMD lane per thread, shared-memory vectors, both
//                          passes, on the second stream
// A forward pass keeps the suboptimal-score rows (KSW_XSUBO) in global scratch; with
// KSW_XSTART the same pass then runs over the reversed query and target prefixes.

#include <algorithm>
#include <cstring>
#include <vector>

#include "bsb_internal.cuh"
#include "sw_pack.cuh"

namespace {

using namespace bsbsw;

constexpr int kSwBlock = 64;

struct SwParams {
    int8_t mat[25];
    int o_del, e_del, o_ins, e_ins;
    int shift, qmax;       // ksw_qinit's shift (uint8) and max (the largest score, >= 1)
    int slen8, slen16;     // segments per lane of the longest byte-lane and word-lane queries
};

template <int P>
__device__ __forceinline__ unsigned grp_mask(int lane)
{
    return ((1u << P) - 1) << (lane & ~(P - 1) & 31);
}

template <int P>
__device__ __forceinline__ int grp_max(unsigned m, int v)
{
#pragma unroll
    for (int d = P / 2; d > 0; d >>= 1) v = max(v, __shfl_xor_sync(m, v, d, P));
    return v;
}

template <int P>
__device__ __forceinline__ int grp_min(unsigned m, int v)
{
#pragma unroll
    for (int d = P / 2; d > 0; d >>= 1) v = min(v, __shfl_xor_sync(m, v, d, P));
    return v;
}

__device__ __forceinline__ int sat8(int x) { return x < 0 ? 0 : x > 255 ? 255 : x; }
__device__ __forceinline__ int sat16(int x) { return x < -32768 ? -32768 : x > 32767 ? 32767 : x; }
__device__ __forceinline__ int subs16(int a, int b)          // _mm_subs_epu16 on values read as uint16
{
    const int d = (int)(uint16_t)a - (int)(uint16_t)b;
    return (int16_t)(uint16_t)(d < 0 ? 0 : d);
}

// One ksw_u8 (P = 16) or ksw_i16 (P = 8) pass (ksw.c:98-327) of the group.  q(c) and t(i)
// give query column c (< qlen) and target row i.  The caller's vectors hold slen*P entries.
// b (P = 16 or 8, XSUBO only) receives the rows of the suboptimal-score bookkeeping.
template <int P, class Q, class T>
__device__ PassOut sw_pass(const SwParams &S, const int8_t *smat, int qlen, int tlen, const Q &q, const T &t, int xtra,
                           int16_t *H0, int16_t *H1, int16_t *E, int16_t *Hmax, uint8_t *qs, int2 *bbuf, int lane,
                           unsigned gm)
{
    constexpr bool U8 = P == 16;
    const int l = lane & (P - 1);
    const int slen = (qlen + P - 1) / P, n = slen * P;
    const int minsc = (xtra & kXSubo) ? xtra & 0xffff : 0x10000;
    const int endsc = (xtra & kXStop) ? xtra & 0xffff : 0x10000;
    // the penalties as the reference broadcasts them (_mm_set1_epi8 / _mm_set1_epi16)
    const int oe_del = S.o_del + S.e_del, oe_ins = S.o_ins + S.e_ins;
    const int pe_del = U8 ? (uint8_t)S.e_del : (uint16_t)S.e_del, poe_del = U8 ? (uint8_t)oe_del : (uint16_t)oe_del;
    const int pe_ins = U8 ? (uint8_t)S.e_ins : (uint16_t)S.e_ins, poe_ins = U8 ? (uint8_t)oe_ins : (uint16_t)oe_ins;
    const int shift = S.shift;
    for (int x = l; x < n; x += P) {       // ksw_qinit's striping; the vectors start at zero
        const int j = x / P, c = j + (x % P) * slen;
        qs[x] = c < qlen ? (uint8_t)q(c) : 0xff;
        H0[x] = 0, E[x] = 0, Hmax[x] = 0;
    }
    __syncwarp(gm);
    PassOut r;
    r.score = 0, r.te = -1, r.qe = -1, r.score2 = -1, r.te2 = -1;
    int gmax = 0, te = -1, n_b = 0, last_row = -2, last_sc = 0;
    for (int i = 0; i < tlen; ++i) {
        const int tc = t(i);
        const int8_t *srow = smat + tc * 5;
        int h = __shfl_up_sync(gm, slen ? (int)H0[(slen - 1) * P + l] : 0, 1, P);   // H(i-1, -1), ksw.c:141-142
        if (l == 0) h = 0;
        int f = 0, mx = 0;
        for (int j = 0; j < slen; ++j) {
            const int x = j * P + l;
            const int qc = qs[x];
            int s = qc == 0xff ? 0 : srow[qc];
            int hv;
            if (U8) hv = sat8(sat8(h + (uint8_t)(s + shift)) - shift);
            else hv = sat16(h + s);
            const int e = E[x];
            hv = max(hv, e);
            hv = max(hv, f);
            mx = max(mx, hv);
            H1[x] = (int16_t)hv;
            if (U8) {
                E[x] = (int16_t)max(sat8(e - pe_del), sat8(hv - poe_del));
                f = max(sat8(f - pe_ins), sat8(hv - poe_ins));
            } else {
                E[x] = (int16_t)max(subs16(e, pe_del), subs16(hv, poe_del));
                f = max(subs16(f, pe_ins), subs16(hv, poe_ins));
            }
            h = H0[x];
        }
        // lazy F (ksw.c:166-177, 284-295).  The reference shifts f up one lane per round and
        // sweeps the segments until no lane can raise an H any more.  The sweep raises H(l, j)
        // to relu(G(l) - j*e_ins) at most, where G(l) is the F arriving at lane l's first column,
        //   G(0) = 0,  G(l) = max(x(l), relu(G(l-1) - slen*e_ins)),  x(l) = the f leaving lane l-1,
        // and its early exit (Farrar's) leaves out only updates that change nothing.  So: the
        // reference's own first test, and where a lane fails it, G as a max-plus scan over the
        // lanes and one max per segment, with no per-segment vote.
        // That bound needs oe_ins >= e_ins as the lanes hold them; byte lanes wrap o_ins + e_ins
        // modulo 256, and there the reference's loop runs as it is.
        if (poe_ins < pe_ins) {
            for (int k = 0; k < 16; ++k) {
                f = __shfl_up_sync(gm, f, 1, P);
                if (l == 0) f = 0;
                bool go = true;
                for (int j = 0; j < slen && go; ++j) {
                    const int x = j * P + l;
                    int hv = max((int)H1[x], f);
                    H1[x] = (int16_t)hv;
                    if (U8) hv = sat8(hv - poe_ins), f = sat8(f - pe_ins);
                    else hv = subs16(hv, poe_ins), f = subs16(f, pe_ins);
                    go = __any_sync(gm, f > hv);
                }
                if (!go) break;
            }
        } else {
            f = __shfl_up_sync(gm, f, 1, P);
            if (l == 0) f = 0;
            if (slen) {
                const int h0 = max((int)H1[l], f);
                const int hh = U8 ? sat8(h0 - poe_ins) : subs16(h0, poe_ins);
                const int fn = U8 ? sat8(f - pe_ins) : subs16(f, pe_ins);
                if (__any_sync(gm, fn > hh)) {
                    const int d = pe_ins * slen;
                    int g = f;
#pragma unroll
                    for (int o = 1; o < P; o <<= 1) {
                        const int v = __shfl_up_sync(gm, g, o, P);
                        if (l >= o) g = max(g, v - o * d);
                    }
                    for (int j = 0; j < slen; ++j, g = max(g - pe_ins, 0)) {
                        const int x = j * P + l;
                        H1[x] = (int16_t)max((int)H1[x], g);
                    }
                } else {
                    H1[l] = (int16_t)h0;
                }
            }
        }
        __syncwarp(gm);
        const int imax = grp_max<P>(gm, mx);
        if (imax >= minsc) {                 // the rows of the suboptimal score (ksw.c:182-189)
            if (n_b == 0 || last_row + 1 != i) {
                if (l == 0) bbuf[n_b] = make_int2(imax, i);
                ++n_b, last_row = i, last_sc = imax;
            } else if (last_sc < imax) {
                if (l == 0) bbuf[n_b - 1] = make_int2(imax, i);
                last_row = i, last_sc = imax;
            }
        }
        if (imax > gmax) {
            gmax = imax, te = i;
            for (int x = l; x < n; x += P) Hmax[x] = H1[x];
            if ((U8 && gmax + shift >= 255) || gmax >= endsc) break;
        }
        int16_t *tmp = H0;
        H0 = H1, H1 = tmp;
        __syncwarp(gm);
    }
    __syncwarp(gm);
    r.score = U8 ? (gmax + shift < 255 ? gmax : 255) : gmax;
    r.te = te;
    if (!U8 || r.score != 255) {
        // qe: the smallest column holding the best Hmax value (ksw.c:196-199)
        int best = -1, col = 0x7fffffff;
        for (int j = 0; j < slen; ++j) {
            const int v = U8 ? (int)Hmax[j * P + l] : (int)(uint16_t)Hmax[j * P + l];
            const int c = j + l * slen;
            if (v > best || (v == best && c < col)) best = v, col = c;
        }
        const int gbest = grp_max<P>(gm, best);
        r.qe = grp_min<P>(gm, best == gbest ? col : 0x7fffffff);
        if (n_b) {                                   // ksw.c:200-207: the first best row outside te +- d
            const int d = (r.score + S.qmax - 1) / S.qmax, low = te - d, high = te + d;
            int bs = -1, bk = 0x7fffffff;
            for (int k = l; k < n_b; k += P) {
                const int2 e = bbuf[k];
                if ((e.y < low || e.y > high) && e.x > bs) bs = e.x, bk = k;
            }
            const int gbs = grp_max<P>(gm, bs);
            const int gk = grp_min<P>(gm, bs == gbs ? bk : 0x7fffffff);
            if (gbs > r.score2 && gk != 0x7fffffff) r.score2 = gbs, r.te2 = bbuf[gk].y;
        }
    }
    return r;
}

struct SeqQ {
    const uint8_t *q;
    __device__ int operator()(int c) const { return q[c]; }
};
struct SeqT {
    const uint8_t *t;
    __device__ int operator()(int i) const { return t[i]; }
};
struct RevQ {                    // query[0..qe] reversed (ksw.c:350)
    const uint8_t *q;
    int qe;
    __device__ int operator()(int c) const { return q[qe - c]; }
};
struct RevT {                    // target[0..te] reversed, the rest as is (ksw.c:350)
    const uint8_t *t;
    int te;
    __device__ int operator()(int i) const { return t[i <= te ? te - i : i]; }
};

template <int P>
__global__ void __launch_bounds__(kSwBlock)
sw_kernel(SwParams S, const bsb_sw_job_t *__restrict__ jobs, const uint8_t *__restrict__ seq,
          const int32_t *__restrict__ list, int total, int *__restrict__ next,
          const int64_t *__restrict__ boff, int2 *__restrict__ bscratch, bsb_kswr_t *__restrict__ out)
{
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ int8_t smat[25];
    if (threadIdx.x < 25) smat[threadIdx.x] = S.mat[threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, l = lane & (P - 1);
    const unsigned gm = grp_mask<P>(lane);
    const int slen_max = P == 16 ? S.slen8 : S.slen16, nv = slen_max * P;
    // per group: H0, H1, E, Hmax (int16) and the striped query (bytes)
    unsigned char *g = sm + (size_t)(threadIdx.x / P) * (size_t)(nv * 9 + 16);
    int16_t *H0 = (int16_t *)g, *H1 = H0 + nv, *E = H1 + nv, *Hmax = E + nv;
    uint8_t *qs = (uint8_t *)(Hmax + nv);
    for (;;) {
        int k = 0;
        if (l == 0) k = atomicAdd(next, 1);
        k = __shfl_sync(gm, k, 0, P);
        if (k >= total) break;
        const int id = list[k];
        const bsb_sw_job_t jb = jobs[id];
        const uint8_t *q = seq + jb.qoff, *t = seq + jb.toff;
        int2 *bbuf = bscratch + boff[id];
        PassOut r = sw_pass<P>(S, smat, jb.qlen, jb.tlen, SeqQ{q}, SeqT{t}, jb.xtra, H0, H1, E, Hmax, qs, bbuf, lane,
                               gm);
        bsb_kswr_t o;
        o.score = r.score, o.te = r.te, o.qe = r.qe, o.score2 = r.score2, o.te2 = r.te2, o.tb = -1, o.qb = -1;
        const bool start = (jb.xtra & kXStart) && !((jb.xtra & kXSubo) && r.score < (jb.xtra & 0xffff));
        // a saturated byte pass leaves qe at -1, where the reference would profile no columns
        if (start && r.qe >= 0) {
            const PassOut rr = sw_pass<P>(S, smat, r.qe + 1, jb.tlen, RevQ{q, r.qe}, RevT{t, r.te}, kXStop | r.score,
                                          H0, H1, E, Hmax, qs, bbuf, lane, gm);
            if (r.score == rr.score) o.tb = r.te - rr.te, o.qb = r.qe - rr.qe;
        }
        if (l == 0) out[id] = o;
        __syncwarp(gm);
    }
}

}  // namespace

extern "C" int bsb_align2_batch(bsb_ctx *ctx, const bsb_ext_param_t *p, const bsb_sw_job_t *jobs, int64_t n,
                                const uint8_t *seq, int64_t seq_bytes, bsb_kswr_t *out)
{
    if (!ctx) return BSB_EINVAL;
    return bsb_align2_run(ctx, p, jobs, n, seq, seq_bytes, out, &ctx->d_in, &ctx->d_in_bytes, &ctx->d_out,
                          &ctx->d_out_bytes);
}

int bsb_align2_run(bsb_ctx *ctx, const bsb_ext_param_t *p, const bsb_sw_job_t *jobs, int64_t n, const uint8_t *seq,
                   int64_t seq_bytes, bsb_kswr_t *out, void **in_buf, size_t *in_bytes, void **out_buf,
                   size_t *out_bytes)
{
    if (!ctx) return BSB_EINVAL;
    if (!p || n < 0 || (n > 0 && (!jobs || !out)) || seq_bytes < 0 || (seq_bytes > 0 && !seq))
        return bsb_fail(ctx, BSB_EINVAL, "NULL argument");
    if (p->e_del < 0 || p->e_ins < 0 || p->o_del < 0 || p->o_ins < 0 || p->o_del > 65535 || p->o_ins > 65535 ||
        p->e_del > 65535 || p->e_ins > 65535)
        return bsb_fail(ctx, BSB_EINVAL, "gap penalties must lie in [0, 65535]");
    SwParams S;
    memcpy(S.mat, p->mat, 25);
    S.o_del = p->o_del, S.e_del = p->e_del, S.o_ins = p->o_ins, S.e_ins = p->e_ins;
    {   // ksw_qinit (ksw.c:66-74) with its uint8 fields
        uint8_t shift = 127, mdiff = 0;
        for (int a = 0; a < 25; ++a) {
            if (p->mat[a] < (int8_t)shift) shift = (uint8_t)p->mat[a];
            if (p->mat[a] > (int8_t)mdiff) mdiff = (uint8_t)p->mat[a];
        }
        S.qmax = mdiff;
        S.shift = (uint8_t)(256 - shift);
    }
    if (S.qmax < 1) return bsb_fail(ctx, BSB_EINVAL, "the scoring matrix needs a positive entry");
    if (n == 0) return 0;
    if (n > 0x7fffffff) return bsb_fail(ctx, BSB_EINVAL, "at most 2^31 - 1 jobs per call");
    {
        int rc0;
        if ((rc0 = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc0;
    }
    // Four job lists: packed byte lanes (1..16 segments), packed word lanes (1..40 segments, when
    // 16-bit arithmetic without saturation is exact: qlen * max score <= 32640 and penalties
    // below 32768), then the one-lane byte and word jobs.  The packed lists are in counting-sort
    // order by segment count and then target length, both descending.
    constexpr int kLenBins = 64, kKeys8 = kPackMaxSeg8 * kLenBins, kKeys16 = kPackMaxSeg16 * kLenBins;
    const bool w16_ok = S.o_del + S.e_del <= 32767 && S.o_ins + S.e_ins <= 32767;
    // the packed passes read F in closed form, which needs oe_ins >= e_ins as the lanes hold them
    const bool b8_ok = (uint8_t)(S.o_ins + S.e_ins) >= (uint8_t)S.e_ins;
    std::vector<int64_t> boff((size_t)n);
    std::vector<int32_t> key((size_t)n);
    std::vector<int32_t> lists((size_t)n);
    std::vector<int64_t> kcnt((size_t)(kKeys8 + kKeys16) + 1, 0);
    int64_t nb = 0, n_fb8 = 0, n_fb16 = 0, n_p8 = 0, n_p16 = 0;
    int max8 = 0, max16 = 0;
    for (int64_t i = 0; i < n; ++i) {
        const bsb_sw_job_t &j = jobs[i];
        if (j.qlen < 0 || j.tlen < 0 || j.qoff < 0 || j.toff < 0 || j.qoff > seq_bytes - j.qlen ||
            j.toff > seq_bytes - j.tlen)
            return bsb_fail(ctx, BSB_EINVAL, "job %lld: bytes outside seq", (long long)i);
        if (j.qlen > BSB_SW_MAX_QLEN)
            return bsb_fail(ctx, BSB_ETOOLONG, "job %lld: qlen %d > %d", (long long)i, j.qlen, BSB_SW_MAX_QLEN);
        boff[(size_t)i] = nb;
        if (j.xtra & kXSubo) nb += j.tlen;
        const int bin = kLenBins - 1 - std::min(j.tlen >> 4, kLenBins - 1);
        const bool byte = j.xtra & kXByte;
        const int sl = byte ? (j.qlen + 15) >> 4 : (j.qlen + 7) >> 3;
        int k = -1;
        if (byte && b8_ok && sl >= 1 && sl <= kPackMaxSeg8)
            k = (kPackMaxSeg8 - sl) * kLenBins + bin, ++n_p8;
        else if (!byte && w16_ok && sl >= 1 && sl <= kPackMaxSeg16 && (int64_t)j.qlen * S.qmax <= 32640)
            k = kKeys8 + (kPackMaxSeg16 - sl) * kLenBins + bin, ++n_p16;
        else if (byte)
            ++n_fb8, max8 = std::max(max8, j.qlen);
        else
            ++n_fb16, max16 = std::max(max16, j.qlen);
        key[(size_t)i] = k;
        if (k >= 0) ++kcnt[(size_t)k + 1];
    }
    for (int k = 0; k < kKeys8 + kKeys16; ++k) kcnt[(size_t)k + 1] += kcnt[(size_t)k];
    {   // lists: [packed byte | packed word | one-lane byte | one-lane word]
        int64_t p8 = n_p8 + n_p16, p16 = n_p8 + n_p16 + n_fb8;
        for (int64_t i = 0; i < n; ++i) {
            const int k = key[(size_t)i];
            if (k >= 0) lists[(size_t)kcnt[(size_t)k]++] = (int32_t)i;
            else if (jobs[i].xtra & kXByte) lists[(size_t)p8++] = (int32_t)i;
            else lists[(size_t)p16++] = (int32_t)i;
        }
    }
    S.slen8 = std::max(1, (max8 + 15) / 16), S.slen16 = std::max(1, (max16 + 7) / 8);
    PackParams P8, P16;
    {
        const uint8_t sh = (uint8_t)S.shift;
        for (int tc = 0; tc < 5; ++tc) {
            uint8_t b[8], w[8];
            for (int qc = 0; qc < 5; ++qc) {               // ksw_qinit (ksw.c:80-95)
                b[qc] = (uint8_t)(p->mat[tc * 5 + qc] + sh);
                w[qc] = (uint8_t)p->mat[tc * 5 + qc];
            }
            b[5] = sh, w[5] = 0;                           // the padding column: score 0
            P8.plo[tc] = (uint32_t)b[0] | (uint32_t)b[1] << 8 | (uint32_t)b[2] << 16 | (uint32_t)b[3] << 24;
            P8.phi[tc] = (uint32_t)b[4] | (uint32_t)b[5] << 8;
            P16.plo[tc] = (uint32_t)w[0] | (uint32_t)w[1] << 8 | (uint32_t)w[2] << 16 | (uint32_t)w[3] << 24;
            P16.phi[tc] = (uint32_t)w[4];
        }
        // the penalties as _mm_set1_epi8 / _mm_set1_epi16 broadcast them, negated in both halves
        P8.nshift = neg2(S.shift);
        P8.npe_del = neg2((uint8_t)S.e_del), P8.npoe_del = neg2((uint8_t)(S.o_del + S.e_del));
        P8.npe_ins = neg2((uint8_t)S.e_ins), P8.npoe_ins = neg2((uint8_t)(S.o_ins + S.e_ins));
        P8.shift = S.shift, P8.qmax = S.qmax, P8.pe_ins = (uint8_t)S.e_ins;
        P16.nshift = 0;
        P16.npe_del = neg2(std::min(S.e_del, 32767)), P16.npoe_del = neg2(std::min(S.o_del + S.e_del, 32767));
        P16.npe_ins = neg2(std::min(S.e_ins, 32767)), P16.npoe_ins = neg2(std::min(S.o_ins + S.e_ins, 32767));
        P16.shift = 0, P16.qmax = S.qmax, P16.pe_ins = std::min(S.e_ins, 32767);
    }
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    cudaStream_t st = ctx->stream;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t jb = al(sizeof(bsb_sw_job_t) * (size_t)n), sb = al((size_t)seq_bytes), ob = al(8 * (size_t)n);
    const size_t lb = al(sizeof(int32_t) * (size_t)n);
    if ((rc = bsb_ensure(ctx, in_buf, in_bytes, jb + sb + ob + lb + 256, "SW input staging"))) return rc;
    char *in = (char *)*in_buf;
    bsb_sw_job_t *d_jobs = (bsb_sw_job_t *)in;
    uint8_t *d_seq = (uint8_t *)(in + jb);
    int64_t *d_boff = (int64_t *)(in + jb + sb);
    int32_t *d_list = (int32_t *)(in + jb + sb + ob);
    const size_t bb = al(sizeof(int2) * (size_t)(nb > 0 ? nb : 1)), rb = al((size_t)n);
    constexpr size_t kCtrBytes = 4096;
    if ((rc = bsb_ensure(ctx, &ctx->arena2, &ctx->arena2_bytes, lb + rb + kCtrBytes + bb, "SW scratch"))) return rc;
    char *a2 = (char *)ctx->arena2;
    int32_t *d_rlist = (int32_t *)a2;                   // reverse lists: byte jobs, then word jobs
    uint8_t *d_rsl = (uint8_t *)(a2 + lb);
    // counters: [0..1] one-lane queues, then one block of kCtrInts per packed lane width
    int *cnt = (int *)(a2 + lb + rb);
    int *ctr8 = cnt + 64, *ctr16 = cnt + 64 + kCtrInts;
    int2 *d_b = (int2 *)(a2 + lb + rb + kCtrBytes);
    if ((rc = bsb_ensure(ctx, out_buf, out_bytes, sizeof(bsb_kswr_t) * (size_t)n + 256, "SW output"))) return rc;
    bsb_kswr_t *d_out = (bsb_kswr_t *)*out_buf;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(d_jobs, jobs, sizeof(bsb_sw_job_t) * n, cudaMemcpyHostToDevice, st),
                       "H2D jobs")) ||
        (seq_bytes && (rc = bsb_cuda(ctx, cudaMemcpyAsync(d_seq, seq, seq_bytes, cudaMemcpyHostToDevice, st), "H2D seq"))) ||
        (rc = bsb_cuda(ctx, cudaMemcpyAsync(d_boff, boff.data(), 8 * n, cudaMemcpyHostToDevice, st), "H2D offsets")) ||
        (rc = bsb_cuda(ctx, cudaMemcpyAsync(d_list, lists.data(), 4 * n, cudaMemcpyHostToDevice, st), "H2D lists")) ||
        (rc = bsb_cuda(ctx, cudaMemsetAsync(cnt, 0, kCtrBytes, st), "SW counters")))
        return rc;
    // the word-lane and one-lane jobs on a second stream, beside the packed byte-lane jobs
    const bool side = n_p16 + n_fb8 + n_fb16 > 0;
    cudaStream_t st2 = ctx->ms.aux[0];
    if (side) {
        if ((rc = bsb_cuda(ctx, cudaEventRecord(ctx->ms.fork, st), "SW fork")) ||
            (rc = bsb_cuda(ctx, cudaStreamWaitEvent(st2, ctx->ms.fork, 0), "SW fork")))
            return rc;
        if (n_p16) {   // word lanes: the 17..40-segment part of the list, then the 1..16 part
            const int32_t *l16 = d_list + n_p8;
            int32_t *r16 = d_rlist + n_p8;
            const int n_hi = (int)(kcnt[(size_t)(kKeys8 + (kPackMaxSeg16 - 16) * kLenBins - 1)] - n_p8), n16 = (int)n_p16;
            if ((rc = bsb_cuda(ctx, sw_pack16_run_hi(false, P16, d_jobs, d_seq, l16, n_hi, d_boff, d_b, d_out, d_rsl,
                                                     ctr16, 0, ctx->n_sm, st2), "SW word-lane kernels")) ||
                (rc = bsb_cuda(ctx, sw_pack16_run_lo(false, P16, d_jobs, d_seq, l16 + n_hi, n16 - n_hi, d_boff, d_b,
                                                     d_out, d_rsl, ctr16, 1, ctx->n_sm, st2), "SW word-lane kernels")))
                return rc;
            sw_rev_scatter<kPackMaxSeg16><<<(int)std::min<int64_t>((n16 + 255) / 256, (int64_t)ctx->n_sm * 4), 256,
                                            0, st2>>>(l16, n16, d_rsl, ctr16, r16);
            if ((rc = bsb_cuda(ctx, sw_pack16_run_hi(true, P16, d_jobs, d_seq, r16, n16, d_boff, d_b, d_out, d_rsl,
                                                     ctr16, 2, ctx->n_sm, st2), "SW word-lane kernels")) ||
                (rc = bsb_cuda(ctx, sw_pack16_run_lo(true, P16, d_jobs, d_seq, r16, n16, d_boff, d_b, d_out, d_rsl,
                                                     ctr16, 3, ctx->n_sm, st2), "SW word-lane kernels")))
                return rc;
        }
        // shared memory per group: 4 int16 vectors + the striped query, slen*P entries each
        const size_t sm8 = (size_t)(kSwBlock / 16) * (size_t)(S.slen8 * 16 * 9 + 16);
        const size_t sm16 = (size_t)(kSwBlock / 8) * (size_t)(S.slen16 * 8 * 9 + 16);
        static bool attr_set = false;
        if (!attr_set) {
            cudaFuncSetAttribute(sw_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
            cudaFuncSetAttribute(sw_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
            attr_set = true;
        }
        const int blocks = ctx->n_sm * 16;
        const int32_t *fb = d_list + n_p8 + n_p16;
        if (n_fb8)
            sw_kernel<16><<<(int)std::min<int64_t>(blocks, (n_fb8 + 3) / 4), kSwBlock, sm8, st2>>>(
                S, d_jobs, d_seq, fb, (int)n_fb8, cnt + 0, d_boff, d_b, d_out);
        if (n_fb16)
            sw_kernel<8><<<(int)std::min<int64_t>(blocks, (n_fb16 + 7) / 8), kSwBlock, sm16, st2>>>(
                S, d_jobs, d_seq, fb + n_fb8, (int)n_fb16, cnt + 1, d_boff, d_b, d_out);
        if ((rc = bsb_cuda(ctx, cudaGetLastError(), "SW one-lane kernels")) ||
            (rc = bsb_cuda(ctx, cudaEventRecord(ctx->ms.join[0], st2), "SW join")))
            return rc;
    }
    if (n_p8) {        // byte lanes: forward passes, grouping by reversed segment count, reverse passes
        const int n8 = (int)n_p8;
        if ((rc = bsb_cuda(ctx, sw_pack_run<16, 1, kPackMaxSeg8, kPackMaxSeg8>(false, P8, d_jobs, d_seq, d_list, n8,
                                                                               d_boff, d_b, d_out, d_rsl, ctr8, 0,
                                                                               ctx->n_sm, st), "SW byte-lane kernels")))
            return rc;
        sw_rev_scatter<kPackMaxSeg8><<<(int)std::min<int64_t>((n8 + 255) / 256, (int64_t)ctx->n_sm * 4), 256, 0,
                                       st>>>(d_list, n8, d_rsl, ctr8, d_rlist);
        if ((rc = bsb_cuda(ctx, sw_pack_run<16, 1, kPackMaxSeg8, kPackMaxSeg8>(true, P8, d_jobs, d_seq, d_rlist, n8,
                                                                               d_boff, d_b, d_out, d_rsl, ctr8, 1,
                                                                               ctx->n_sm, st), "SW byte-lane kernels")))
            return rc;
    }
    if (side && (rc = bsb_cuda(ctx, cudaStreamWaitEvent(st, ctx->ms.join[0], 0), "SW join"))) return rc;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(out, d_out, sizeof(bsb_kswr_t) * n, cudaMemcpyDeviceToHost, st), "D2H")))
        return rc;
    return bsb_cuda(ctx, cudaStreamSynchronize(st), "SW batch");
}
