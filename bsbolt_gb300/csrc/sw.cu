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
//   sw_partition    byte-lane and word-lane jobs into two lists
//   sw_kernel<16>   byte-lane jobs (ksw_u8), two jobs per warp
//   sw_kernel<8>    word-lane jobs (ksw_i16), four jobs per warp
// Each job: the forward pass with the suboptimal-score rows (KSW_XSUBO) kept in global
// scratch, then, with KSW_XSTART, the same pass over the reversed query and target prefixes.

#include <algorithm>
#include <cstring>
#include <vector>

#include "bsb_internal.cuh"

namespace {

constexpr int kSwBlock = 64;
constexpr int kXByte = 0x10000, kXStop = 0x20000, kXSubo = 0x40000, kXStart = 0x80000;

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

struct PassOut {
    int score, te, qe, score2, te2;
};

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
        // lazy F (ksw.c:166-177, 284-295): each round shifts f up one lane
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

__global__ void sw_partition(const bsb_sw_job_t *__restrict__ jobs, int64_t n, int *__restrict__ cnt,
                             int32_t *__restrict__ list8, int32_t *__restrict__ list16)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (jobs[i].xtra & kXByte) list8[atomicAdd(&cnt[0], 1)] = (int32_t)i;
        else list16[atomicAdd(&cnt[1], 1)] = (int32_t)i;
    }
}

template <int P>
__global__ void __launch_bounds__(kSwBlock)
sw_kernel(SwParams S, const bsb_sw_job_t *__restrict__ jobs, const uint8_t *__restrict__ seq,
          const int32_t *__restrict__ list, const int *__restrict__ n_list, int *__restrict__ next,
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
    const int total = *n_list;
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
    int max8 = 0, max16 = 0;
    std::vector<int64_t> boff((size_t)n);
    int64_t nb = 0;
    for (int64_t i = 0; i < n; ++i) {
        const bsb_sw_job_t &j = jobs[i];
        if (j.qlen < 0 || j.tlen < 0 || j.qoff < 0 || j.toff < 0 || j.qoff > seq_bytes - j.qlen ||
            j.toff > seq_bytes - j.tlen)
            return bsb_fail(ctx, BSB_EINVAL, "job %lld: bytes outside seq", (long long)i);
        if (j.qlen > BSB_SW_MAX_QLEN)
            return bsb_fail(ctx, BSB_ETOOLONG, "job %lld: qlen %d > %d", (long long)i, j.qlen, BSB_SW_MAX_QLEN);
        if (j.xtra & kXByte) max8 = std::max(max8, j.qlen);
        else max16 = std::max(max16, j.qlen);
        boff[(size_t)i] = nb;
        if (j.xtra & kXSubo) nb += j.tlen;
    }
    S.slen8 = std::max(1, (max8 + 15) / 16), S.slen16 = std::max(1, (max16 + 7) / 8);
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    cudaStream_t st = ctx->stream;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t jb = al(sizeof(bsb_sw_job_t) * (size_t)n), sb = al((size_t)seq_bytes), ob = al(8 * (size_t)n);
    if ((rc = bsb_ensure(ctx, &ctx->d_in, &ctx->d_in_bytes, jb + sb + ob + 256, "SW input staging"))) return rc;
    char *in = (char *)ctx->d_in;
    bsb_sw_job_t *d_jobs = (bsb_sw_job_t *)in;
    uint8_t *d_seq = (uint8_t *)(in + jb);
    int64_t *d_boff = (int64_t *)(in + jb + sb);
    const size_t lb = al(sizeof(int32_t) * (size_t)n), bb = al(sizeof(int2) * (size_t)(nb > 0 ? nb : 1));
    if ((rc = bsb_ensure(ctx, &ctx->arena2, &ctx->arena2_bytes, 2 * lb + 256 + bb, "SW scratch"))) return rc;
    char *a2 = (char *)ctx->arena2;
    int32_t *list8 = (int32_t *)a2, *list16 = (int32_t *)(a2 + lb);
    int *cnt = (int *)(a2 + 2 * lb);                    // [0..1] list sizes, [2..3] queue heads
    int2 *d_b = (int2 *)(a2 + 2 * lb + 256);
    if ((rc = bsb_ensure(ctx, &ctx->d_out, &ctx->d_out_bytes, sizeof(bsb_kswr_t) * (size_t)n + 256, "SW output")))
        return rc;
    bsb_kswr_t *d_out = (bsb_kswr_t *)ctx->d_out;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(d_jobs, jobs, sizeof(bsb_sw_job_t) * n, cudaMemcpyHostToDevice, st),
                       "H2D jobs")) ||
        (seq_bytes && (rc = bsb_cuda(ctx, cudaMemcpyAsync(d_seq, seq, seq_bytes, cudaMemcpyHostToDevice, st), "H2D seq"))) ||
        (rc = bsb_cuda(ctx, cudaMemcpyAsync(d_boff, boff.data(), 8 * n, cudaMemcpyHostToDevice, st), "H2D offsets")) ||
        (rc = bsb_cuda(ctx, cudaMemsetAsync(cnt, 0, 4 * sizeof(int), st), "SW counters")))
        return rc;
    const int pb = (int)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->n_sm * 8);
    sw_partition<<<pb, 256, 0, st>>>(d_jobs, n, cnt, list8, list16);
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
    if (max8 > 0)
        sw_kernel<16><<<blocks, kSwBlock, sm8, st>>>(S, d_jobs, d_seq, list8, cnt + 0, cnt + 2, d_boff, d_b, d_out);
    if (max16 > 0)
        sw_kernel<8><<<blocks, kSwBlock, sm16, st>>>(S, d_jobs, d_seq, list16, cnt + 1, cnt + 3, d_boff, d_b, d_out);
    if ((rc = bsb_cuda(ctx, cudaGetLastError(), "SW kernels"))) return rc;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(out, d_out, sizeof(bsb_kswr_t) * n, cudaMemcpyDeviceToHost, st), "D2H")))
        return rc;
    return bsb_cuda(ctx, cudaStreamSynchronize(st), "SW batch");
}
