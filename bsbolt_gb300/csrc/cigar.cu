// cigar.cu -- bwa_gen_cigar2 (bsbolt/External/BWA/bwa.c:199-351) for batches of
// alignments on sm_103a: the banded global alignment with traceback (ksw_global2,
// ksw.c:504-606), the CIGAR, and the MD / XB strings with the methylation counts.
//
// One warp per alignment.  The warp stages the job's sequences into its slice of
// shared memory (query and reference after the strand flip of bwa.c:217-221, the
// original read and the 2-base-padded original reference after bwa.c:267-271),
// reading the device pac / opac directly; the ungapped score (bwa.c:222-230) is a
// warp sum.  What the reference does as one sequential pass -- the DP rows with
// their F chain, the traceback, and the MD / XB text whose run lengths carry from
// base to base -- runs on lane 0 out of shared memory.  The bands mem_reg2aln asks
// for are narrow (infer_bw, bwamem.c:1219-1223: 0 for a near-perfect ungapped hit,
// a few columns per indel), so these passes are a few hundred steps.  Jobs longer
// than kSmemLen keep their arrays in global scratch instead.
//
//   plan_kernel       per job: reject test, band, sizes of its global scratch and output slot
//   scan x2           scratch and slot offsets (scan.cuh)
//   cigar_kernel      per job (one warp): staging, DP / traceback, CIGAR words, MD / XB
//   scan + compact    packs the records the host reads back

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "bsb_internal.cuh"
#include "ksw_global.cuh"
#include "scan.cuh"

namespace {

constexpr int kCigarBlock = 128;
constexpr int kCigarWarps = kCigarBlock / 32;
constexpr int kUnit = 16;                   // scratch and slot sizes are counted in 16-byte units
constexpr int kSmemLen = 256;               // query and reference intervals up to this stay in shared memory
constexpr int kSmemZ = 2048;                // backtrack bytes held in shared memory
constexpr int kCallsCap = 5 * kSmemLen + 16; // XB calls: at most 5 characters per query base

struct CigarParams {
    int8_t mat[25];
    int o_del, e_del, o_ins, e_ins;
    int64_t l_pac, crick_l;
};

// One warp's shared-memory slice.
struct WarpSmem {
    int32_t H[kSmemLen + 1], E[kSmemLen + 1];
    uint32_t z[kSmemZ / 4];
    uint8_t q[kSmemLen], t[kSmemLen], o[kSmemLen], c[kSmemLen + 4];
    char calls[kCallsCap];
};

__device__ __forceinline__ int pac_at(const uint8_t *__restrict__ pac, int64_t k)     // _get_pac, bntseq.h:79
{
    return pac[k >> 2] >> ((~k & 3) << 1) & 3;
}

// Base at pos of the doubled sequence (bns_get_seq, bntseq.c:413-434, one position).
__device__ __forceinline__ int dseq_at(const uint8_t *__restrict__ pac, int64_t l_pac, int64_t pos)
{
    return pos >= l_pac ? 3 - pac_at(pac, (l_pac << 1) - 1 - pos) : pac_at(pac, pos);
}

__host__ __device__ __forceinline__ int64_t round_unit(int64_t b) { return (b + kUnit - 1) / kUnit * kUnit; }

struct JobPlan {
    bool reject, ungapped, big, z_smem;
    int l, rlen, w, stride;
    // global scratch layout (byte offsets): XB calls, backtrack bytes, then (big jobs) the
    // staged sequences and the H / E rows
    int64_t calls_at, z_at, seq_at, he_at, scratch;
    int slot_units;
};

// The reject test and band of bwa_gen_cigar2 (bwa.c:211-240) for one job, and where its
// arrays live.
__device__ __forceinline__ JobPlan plan_job(const CigarParams &P, const bsb_cigar_job_t &jb)
{
    JobPlan p{};
    const int64_t rb = jb.rb, re = jb.re, lp = P.l_pac;
    p.l = jb.l_query;
    // bwa.c:211, and bns_get_seq clamping [rb, re) to the doubled sequence (bwa.c:214-215)
    p.reject = p.l <= 0 || rb >= re || (rb < lp && re > lp) || rb < 0 || re > 2 * lp;
    if (p.reject) return p;
    p.rlen = (int)(re - rb);
    p.ungapped = p.l == p.rlen && jb.w == 0;
    p.big = p.l > kSmemLen || p.rlen > kSmemLen;
    if (!p.ungapped) {
        const int l = p.l, m0 = P.mat[0];
        const int max_ins = band_cap(((l + 1) >> 1) * m0 - P.o_ins, P.e_ins);
        const int max_del = band_cap(((l + 1) >> 1) * m0 - P.o_del, P.e_del);
        int max_gap = max_ins > max_del ? max_ins : max_del;
        max_gap = max_gap > 1 ? max_gap : 1;
        const int dl = abs(p.rlen - l);
        int w = (max_gap + dl + 1) >> 1;
        w = w < jb.w ? w : jb.w;
        p.w = w > dl + 3 ? w : dl + 3;
        const int n_col = l < 2 * p.w + 1 ? l : 2 * p.w + 1;
        p.stride = (n_col + 3) & ~3;
        p.z_smem = !p.big && (int64_t)p.stride * p.rlen <= kSmemZ;
    }
    int64_t at = 0;
    p.calls_at = at;
    if (p.big) at += round_unit(5 * (int64_t)p.l + 16);
    p.z_at = at;
    if (!p.ungapped && !p.z_smem) at += round_unit((int64_t)p.stride * p.rlen);
    p.seq_at = at;
    if (p.big) at += round_unit(3 * (int64_t)p.l + p.rlen + 4 + p.rlen);
    p.he_at = at;
    if (p.big && !p.ungapped) at += round_unit(8 * (int64_t)(p.l + 1));
    p.scratch = at;
    // CIGAR words (at most one op per base of either sequence) and the MD/XB text
    const int64_t slot = 4 * (int64_t)(p.l + p.rlen + 2) + 10 * (int64_t)(p.l + p.rlen) + 32;
    p.slot_units = (int)((slot + kUnit - 1) / kUnit);
    return p;
}

__global__ void plan_kernel(CigarParams P, const bsb_cigar_job_t *__restrict__ jobs, int n,
                            int *__restrict__ scratch_units, int *__restrict__ slot_units)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const JobPlan p = plan_job(P, jobs[i]);
        scratch_units[i] = p.reject ? 0 : (int)(p.scratch / kUnit);
        slot_units[i] = p.reject ? 0 : p.slot_units;
    }
}

// The traceback of ksw_global2 (ksw.c:584-600), one thread: ops come out last-first, then
// are reversed.  Returns false when a step leaves the band.
__device__ __forceinline__ bool global_traceback(const uint8_t *Z, int qlen, int tlen, int w, int stride, uint32_t *cig,
                                 int &n_cigar)
{
    int which = 0, i = tlen - 1, k = (i + w + 1 < qlen ? i + w + 1 : qlen) - 1;
    n_cigar = 0;
    auto push = [&](int op, int len) {
        if (n_cigar && (int)(cig[n_cigar - 1] & 0xf) == op) cig[n_cigar - 1] += (uint32_t)len << 4;
        else cig[n_cigar++] = (uint32_t)len << 4 | op;
    };
    while (i >= 0 && k >= 0) {
        const int beg = i > w ? i - w : 0, end = i + w + 1 < qlen ? i + w + 1 : qlen;
        if (k < beg || k >= end) return false;
        which = Z[(size_t)i * stride + (k - beg)] >> (which << 1) & 3;
        if (which == 0) push(0, 1), --i, --k;
        else if (which == 1) push(2, 1), --i;
        else push(1, 1), --k;
    }
    if (i >= 0) push(2, i + 1);
    if (k >= 0) push(1, k + 1);
    for (int a = 0; a < n_cigar >> 1; ++a) {
        const uint32_t t = cig[a];
        cig[a] = cig[n_cigar - 1 - a];
        cig[n_cigar - 1 - a] = t;
    }
    return true;
}

__device__ __forceinline__ int ndigits(int v) { return v < 10 ? 1 : v < 100 ? 2 : v < 1000 ? 3 : v < 10000 ? 4 : 5; }

__device__ __forceinline__ void write_int(char *p, int v, int nd)
{
    for (int k = nd - 1; k >= 0; --k) p[k] = (char)('0' + v % 10), v /= 10;
}

// Highest set bit of x below bit `lane`, or -1.
__device__ __forceinline__ int prev_bit(uint32_t x, int lane)
{
    const uint32_t below = x & ((1u << lane) - 1);
    return below ? 31 - __clz(below) : -1;
}

// One job's record (written by one lane).
__device__ __forceinline__ void finish(bsb_cigar_out_t *out, int *bytes, int id, int status, int score, int n_cigar,
                                       int nm, int cg_m, int cg_u, int ch_m, int ch_u, int b)
{
    bsb_cigar_out_t &o = out[id];
    o.score = score, o.n_cigar = n_cigar, o.NM = nm;
    o.cg_meth = cg_m, o.cg_unmeth = cg_u, o.ch_meth = ch_m, o.ch_unmeth = ch_u;
    o.status = status, o.off = 0, o.bytes = b, o.pad_ = 0;
    bytes[id] = b;
}

__global__ void __launch_bounds__(kCigarBlock)
cigar_kernel(CigarParams P, const bsb_cigar_job_t *__restrict__ jobs, int n, const uint8_t *__restrict__ pac,
             const uint8_t *__restrict__ opac, const uint8_t *__restrict__ qbuf, const uint8_t *__restrict__ obuf,
             const int64_t *__restrict__ scratch_off, const int64_t *__restrict__ slot_off,
             uint8_t *__restrict__ scratch, uint8_t *__restrict__ slots, bsb_cigar_out_t *__restrict__ out,
             int *__restrict__ bytes)
{
    __shared__ int8_t smat[25];
    __shared__ WarpSmem wsm[kCigarWarps];
    if (threadIdx.x < 25) smat[threadIdx.x] = P.mat[threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    WarpSmem &S = wsm[threadIdx.x >> 5];
    const int warps = gridDim.x * kCigarWarps;
    for (int id = blockIdx.x * kCigarWarps + (threadIdx.x >> 5); id < n; id += warps) {
        const bsb_cigar_job_t jb = jobs[id];
        const JobPlan p = plan_job(P, jb);
        if (p.reject) {
            if (lane == 0) finish(out, bytes, id, BSB_CIGAR_REJECT, 0, 0, -1, 0, 0, 0, 0, 0);
            continue;
        }
        const int64_t lp = P.l_pac, rb = jb.rb, re = jb.re;
        const int l = p.l, rlen = p.rlen;
        const bool flip = rb >= lp;          // both sequences reversed (bwa.c:217-221)
        const bool reverse = rb > lp;        // bwa.c:212 ('>', unlike the flip)
        const uint8_t *q = qbuf + jb.qoff;
        const uint8_t *oq = obuf + jb.ooff;
        uint8_t *scr = scratch + scratch_off[id] * kUnit;
        uint32_t *cig = reinterpret_cast<uint32_t *>(slots + slot_off[id] * kUnit);
        uint8_t *qs = S.q, *ts = S.t, *os = S.o, *cs = S.c;
        char *calls = S.calls;
        int32_t *H = S.H, *E = S.E;
        uint8_t *Z = reinterpret_cast<uint8_t *>(S.z);
        if (p.big) {
            uint8_t *g = scr + p.seq_at;
            qs = g, ts = g + l, os = g + l + rlen, cs = g + 2 * l + rlen;
            calls = reinterpret_cast<char *>(scr + p.calls_at);
            H = reinterpret_cast<int32_t *>(scr + p.he_at), E = H + (l + 1);
        }
        if (!p.ungapped && !p.z_smem) Z = scr + p.z_at;
        // stage the query and reference (after the flip)
        for (int j = lane; j < l; j += 32) qs[j] = q[flip ? l - 1 - j : j];
        for (int i = lane; i < rlen; i += 32) ts[i] = (uint8_t)dseq_at(pac, lp, flip ? re - 1 - i : rb + i);
        __syncwarp();
        int n_cigar = 0, score = 0, band_exit = 0;
        if (p.ungapped) {                     // bwa.c:222-230
            int sum = 0;
            for (int i = lane; i < l; i += 32) sum += smat[ts[i] * 5 + qs[i]];
            score = __reduce_add_sync(BSB_FULL_MASK, sum);
            n_cigar = 1;
            if (lane == 0) cig[0] = (uint32_t)l << 4;
        } else {                              // ksw_global2: rows on the warp, traceback on lane 0
            score = global_rows_warp(GlobalPen{P.o_del, P.e_del, P.o_ins, P.e_ins}, smat, qs, l, ts, rlen, p.w, p.stride,
                                     H, E, Z, lane);
            if (lane == 0) band_exit = !global_traceback(Z, l, rlen, p.w, p.stride, cig, n_cigar);
        }
        score = __shfl_sync(BSB_FULL_MASK, score, 0);
        n_cigar = __shfl_sync(BSB_FULL_MASK, n_cigar, 0);
        band_exit = __shfl_sync(BSB_FULL_MASK, band_exit, 0);
        if (band_exit) {
            if (lane == 0) finish(out, bytes, id, BSB_CIGAR_BAND_EXIT, score, n_cigar, -1, 0, 0, 0, 0, 0);
            __syncwarp();
            continue;
        }
        // the original reference with two bases of context each side (bwa.c:264-266)
        const int64_t cb = rb - 2, ce = re + 2;
        const int64_t cbc = cb < 0 ? 0 : cb, cec = ce > 2 * lp ? 2 * lp : ce;
        if (!(cbc >= lp || cec <= lp)) {
            if (lane == 0) finish(out, bytes, id, BSB_CIGAR_NO_MD, score, n_cigar, -1, 0, 0, 0, 0, 4 * n_cigar);
            __syncwarp();
            continue;
        }
        if (cbc != cb || cec != ce) {
            if (lane == 0) finish(out, bytes, id, BSB_CIGAR_CLIPPED, score, n_cigar, -1, 0, 0, 0, 0, 0);
            __syncwarp();
            continue;
        }
        // stage the original read and reference (cseq[t], t < rlen + 4, after bwa.c:267-271)
        for (int x = lane; x < l; x += 32) os[x] = oq[flip ? l - 1 - x : x];
        for (int t = lane; t < rlen + 4; t += 32) cs[t] = (uint8_t)dseq_at(opac, lp, flip ? re + 1 - t : cb + t);
        __syncwarp();
        // MD and XB (bwa.c:252-330) on the warp, 32 bases of an M op at a time.  Each lane
        // classifies its base as a match, a mismatch (an MD token: the run u of non-mismatch
        // bases before it, then the base) or a methylation call (an XB token: the run of
        // non-call bases before it when nonzero, then the context letter); the runs come
        // from the lanes' masks and the carried counts, the token places from a warp scan.
        char *md = reinterpret_cast<char *>(cig + n_cigar);
        const bool is_crick = (rb >= P.crick_l && rb < lp) || rb >= P.crick_l + lp;   // bwa.c:256-258
        const int ref_base = is_crick ? 2 : 1, methyl_base = is_crick ? 0 : 3;
        const char *int2base = rb < lp ? "ACGTN" : "TGCAN";
        int md_len = 0, xb_len = 0, u = 0, mp = 0, n_mm = 0, n_gap = 0;
        int cg_m = 0, cg_u = 0, ch_m = 0, ch_u = 0;
        int x = 0, y = 0;
        for (int k = 0; k < n_cigar; ++k) {
            const int op = cig[k] & 0xf, len = cig[k] >> 4;
            if (op == 0) {
                for (int base = 0; base < len; base += 32) {
                    const int i = base + lane;
                    const bool on = i < len;
                    int code = 0;                 // 0 match, 1 mismatch, 2 call
                    char ch = 0;
                    bool cg = false, meth = false;
                    if (on) {
                        const uint8_t *r = cs + y + i;          // r[2] is the reference base
                        const int r2 = r[2], ob = os[x + i];
                        if (r2 == ref_base) {
                            int b1, b2, b3;
                            if (!reverse && !is_crick) b1 = r2, b2 = r[3], b3 = r[4];
                            else if (!reverse) b1 = r[1], b2 = r2, b3 = r[3];
                            else if (!is_crick) b1 = r2, b2 = r[1], b3 = r[0];
                            else b1 = r[3], b2 = r2, b3 = r[1];
                            if (ob == ref_base || ob == methyl_base) {   // getMethylationContext, bwa.c:180-196
                                code = 2;
                                meth = ob == ref_base;
                                cg = b1 == 1 && b2 == 2;
                                const bool chg = !cg && b1 == 1 && b3 == 2;
                                ch = cg ? (meth ? 'X' : 'x') : chg ? (meth ? 'Y' : 'y') : (meth ? 'Z' : 'z');
                            } else {
                                code = 1, ch = int2base[r2];
                            }
                        } else if (ob != r2) {
                            code = 1, ch = int2base[r2];
                        }
                    }
                    const uint32_t mm = __ballot_sync(BSB_FULL_MASK, code == 1);
                    const uint32_t cl = __ballot_sync(BSB_FULL_MASK, code == 2);
                    const int n_on = len - base < 32 ? len - base : 32;
                    int pm = prev_bit(mm, lane), pc = prev_bit(cl, lane);
                    const int u_here = pm >= 0 ? lane - pm - 1 : u + lane;
                    const int mp_here = pc >= 0 ? lane - pc - 1 : mp + lane;
                    const int md_tok = code == 1 ? ndigits(u_here) + 1 : 0;
                    const int xb_tok = code == 2 ? (mp_here > 0 ? ndigits(mp_here) : 0) + 1 : 0;
                    int packed = md_tok << 16 | xb_tok, incl = packed;        // both scans in one
#pragma unroll
                    for (int d = 1; d < 32; d <<= 1) {
                        const int v = __shfl_up_sync(BSB_FULL_MASK, incl, d);
                        if (lane >= d) incl += v;
                    }
                    const int excl = incl - packed;
                    if (code == 1) {
                        char *dst = md + md_len + (excl >> 16);
                        write_int(dst, u_here, md_tok - 1);
                        dst[md_tok - 1] = ch;
                    } else if (code == 2) {
                        char *dst = calls + xb_len + (excl & 0xffff);
                        if (xb_tok > 1) write_int(dst, mp_here, xb_tok - 1);
                        dst[xb_tok - 1] = ch;
                    }
                    const int tot = __shfl_sync(BSB_FULL_MASK, incl, 31);
                    md_len += tot >> 16, xb_len += tot & 0xffff;
                    u = mm ? n_on - 1 - (31 - __clz(mm)) : u + n_on;
                    mp = cl ? n_on - 1 - (31 - __clz(cl)) : mp + n_on;
                    n_mm += __popc(mm);
                    cg_m += __popc(__ballot_sync(BSB_FULL_MASK, code == 2 && meth && cg));
                    ch_m += __popc(__ballot_sync(BSB_FULL_MASK, code == 2 && meth && !cg));
                    cg_u += __popc(__ballot_sync(BSB_FULL_MASK, code == 2 && !meth && cg));
                    ch_u += __popc(__ballot_sync(BSB_FULL_MASK, code == 2 && !meth && !cg));
                }
                x += len, y += len;
            } else if (op == 2) {
                if (k > 0 && k < n_cigar - 1) {              // no MD for a leading or trailing D
                    const int nd = ndigits(u);
                    if (lane == 0) write_int(md + md_len, u, nd), md[md_len + nd] = '^';
                    for (int i = lane; i < len; i += 32) md[md_len + nd + 1 + i] = int2base[cs[y + i + 2]];
                    md_len += nd + 1 + len;
                    u = 0, n_gap += len;
                }
                y += len;
            } else if (op == 1) {
                x += len, n_gap += len, mp += len;
            }
        }
        {
            const int nd = ndigits(u);
            if (lane == 0) write_int(md + md_len, u, nd);
            md_len += nd;
            if (mp > 0) {
                const int nm = ndigits(mp);
                if (lane == 0) write_int(calls + xb_len, mp, nm);
                xb_len += nm;
            }
        }
        __syncwarp();
        // "MD\tXB:Z:" then the calls, then the NUL
        if (lane < 6) md[md_len + lane] = "\tXB:Z:"[lane];
        for (int t = lane; t <= xb_len; t += 32) md[md_len + 6 + t] = t < xb_len ? calls[t] : 0;
        if (lane == 0)
            finish(out, bytes, id, BSB_CIGAR_OK, score, n_cigar, n_mm + n_gap, cg_m, cg_u, ch_m, ch_u,
                   4 * n_cigar + md_len + 6 + xb_len + 1);
        __syncwarp();
    }
}

// One warp per job: its slot's first bytes[i] bytes to blob + off[i].
__global__ void compact_kernel(const uint8_t *__restrict__ slots, const int64_t *__restrict__ slot_off,
                               const int *__restrict__ bytes, const int64_t *__restrict__ off, int n,
                               uint8_t *__restrict__ blob, bsb_cigar_out_t *__restrict__ out)
{
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
        const uint8_t *src = slots + slot_off[i] * kUnit;
        uint8_t *dst = blob + off[i];
        const int b = bytes[i];
        for (int t = lane; t < b; t += 32) dst[t] = src[t];
        if (lane == 0) {
            out[i].off = off[i];
            out[i].bytes = b;
        }
    }
}

}  // namespace

extern "C" int bsb_index_upload_opac(bsb_ctx *ctx, const uint8_t *opac, int64_t l_pac)
{
    if (!ctx) return BSB_EINVAL;
    if (!ctx->has_index) return bsb_fail(ctx, BSB_ENOINDEX, "no index loaded");
    if (!opac || l_pac != ctx->l_pac || l_pac <= 0)
        return bsb_fail(ctx, BSB_EINVAL, "opac of %lld bases for an index of %lld", (long long)l_pac,
                        (long long)ctx->l_pac);
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    if (ctx->idx_opac) cudaFree(ctx->idx_opac);
    ctx->idx_opac = nullptr;
    const size_t pb = (size_t)(l_pac + 3) / 4;
    if ((rc = bsb_cuda(ctx, cudaMalloc(&ctx->idx_opac, pb + 64), "index: opac"))) return rc;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(ctx->idx_opac, opac, pb, cudaMemcpyHostToDevice, ctx->stream),
                       "index: opac upload")))
        return rc;
    return bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "index: opac upload");
}

extern "C" int bsb_gen_cigar_batch(bsb_ctx *ctx, const bsb_align_opt_t *o, int64_t crick_l, int32_t n,
                                   const bsb_cigar_job_t *jobs, const uint8_t *qbuf, int64_t q_bytes,
                                   const uint8_t *obuf, int64_t o_bytes, bsb_cigar_out_t *out, uint8_t *blob,
                                   int64_t blob_cap, int64_t *blob_used)
{
    if (!ctx) return BSB_EINVAL;
    if (!ctx->has_index || !ctx->idx_pac || !ctx->idx_opac)
        return bsb_fail(ctx, BSB_ENOINDEX, "no index with pac and opac loaded");
    if (!o || n < 0 || (n > 0 && (!jobs || !out || !blob_used)) || q_bytes < 0 || o_bytes < 0 || blob_cap < 0)
        return bsb_fail(ctx, BSB_EINVAL, "NULL argument");
    if (o->e_del < 1 || o->e_ins < 1 || o->o_del < 0 || o->o_ins < 0)
        return bsb_fail(ctx, BSB_EINVAL, "unsupported gap penalties");
    if (blob_used) *blob_used = 0;
    if (n == 0) return 0;
    int rc0;
    if ((rc0 = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc0;
    const int64_t lp = ctx->l_pac;
    for (int32_t i = 0; i < n; ++i) {
        const bsb_cigar_job_t &j = jobs[i];
        if (j.l_query > 0) {
            if (j.qoff < 0 || j.qoff > q_bytes - j.l_query || j.ooff < 0 || j.ooff > o_bytes - j.l_query || !qbuf ||
                !obuf)
                return bsb_fail(ctx, BSB_EINVAL, "job %d: query bytes outside the buffers", i);
            if (j.l_query > BSB_CIGAR_MAX_LEN)
                return bsb_fail(ctx, BSB_ETOOLONG, "job %d: l_query %d > %d", i, j.l_query, BSB_CIGAR_MAX_LEN);
        }
        if (j.w < 0) return bsb_fail(ctx, BSB_EINVAL, "job %d: negative band", i);
        const bool reject = j.l_query <= 0 || j.rb >= j.re || (j.rb < lp && j.re > lp) || j.rb < 0 || j.re > 2 * lp;
        if (!reject && j.re - j.rb > BSB_CIGAR_MAX_LEN)
            return bsb_fail(ctx, BSB_ETOOLONG, "job %d: reference interval %lld > %d", i, (long long)(j.re - j.rb),
                            BSB_CIGAR_MAX_LEN);
    }
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    cudaStream_t st = ctx->stream;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    // inputs: jobs, query bytes, original-read bytes
    const size_t jb = al(sizeof(bsb_cigar_job_t) * (size_t)n), qb = al((size_t)q_bytes), ob = al((size_t)o_bytes);
    if ((rc = bsb_ensure(ctx, &ctx->d_in, &ctx->d_in_bytes, jb + qb + ob + 256, "CIGAR input staging"))) return rc;
    char *in = (char *)ctx->d_in;
    bsb_cigar_job_t *d_jobs = (bsb_cigar_job_t *)in;
    uint8_t *d_q = (uint8_t *)(in + jb), *d_o = (uint8_t *)(in + jb + qb);
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(d_jobs, jobs, sizeof(bsb_cigar_job_t) * n, cudaMemcpyHostToDevice, st),
                       "H2D jobs")))
        return rc;
    if (q_bytes && (rc = bsb_cuda(ctx, cudaMemcpyAsync(d_q, qbuf, q_bytes, cudaMemcpyHostToDevice, st), "H2D query")))
        return rc;
    if (o_bytes && (rc = bsb_cuda(ctx, cudaMemcpyAsync(d_o, obuf, o_bytes, cudaMemcpyHostToDevice, st), "H2D read")))
        return rc;
    // plan: per-job sizes and their offsets
    const size_t ib = al(sizeof(int) * (size_t)n), lb = al(sizeof(int64_t) * ((size_t)n + 1));
    const size_t tb = al(sizeof(int64_t) * (size_t)scan_tmp_words(n));
    if ((rc = bsb_ensure(ctx, &ctx->arena2, &ctx->arena2_bytes, 3 * ib + 3 * lb + tb + 256, "CIGAR plan"))) return rc;
    char *pl = (char *)ctx->arena2;
    int *d_scr_units = (int *)pl, *d_slot_units = (int *)(pl + ib), *d_bytes = (int *)(pl + 2 * ib);
    int64_t *d_scr_off = (int64_t *)(pl + 3 * ib), *d_slot_off = (int64_t *)(pl + 3 * ib + lb);
    int64_t *d_off = (int64_t *)(pl + 3 * ib + 2 * lb), *d_tmp = (int64_t *)(pl + 3 * ib + 3 * lb);
    CigarParams P;
    memcpy(P.mat, o->mat, 25);
    P.o_del = o->o_del, P.e_del = o->e_del, P.o_ins = o->o_ins, P.e_ins = o->e_ins;
    P.l_pac = lp, P.crick_l = crick_l;
    const int blocks = (int)std::min<int64_t>(((int64_t)n + kCigarBlock - 1) / kCigarBlock, (int64_t)ctx->n_sm * 16);
    plan_kernel<<<blocks, kCigarBlock, 0, st>>>(P, d_jobs, n, d_scr_units, d_slot_units);
    if ((rc = bsb_cuda(ctx, scan_i32_i64(d_scr_units, n, d_scr_off, d_tmp, st), "CIGAR scratch offsets"))) return rc;
    if ((rc = bsb_cuda(ctx, scan_i32_i64(d_slot_units, n, d_slot_off, d_tmp, st), "CIGAR slot offsets"))) return rc;
    int64_t tot[2] = {0, 0};
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(&tot[0], d_scr_off + n, 8, cudaMemcpyDeviceToHost, st), "D2H sizes")) ||
        (rc = bsb_cuda(ctx, cudaMemcpyAsync(&tot[1], d_slot_off + n, 8, cudaMemcpyDeviceToHost, st), "D2H sizes")) ||
        (rc = bsb_cuda(ctx, cudaStreamSynchronize(st), "CIGAR plan")))
        return rc;
    const size_t scr_b = al((size_t)tot[0] * kUnit + kUnit), slot_b = al((size_t)tot[1] * kUnit + kUnit);
    if ((rc = bsb_ensure(ctx, &ctx->arena0, &ctx->arena0_bytes, scr_b + slot_b, "CIGAR scratch"))) return rc;
    uint8_t *d_scr = (uint8_t *)ctx->arena0, *d_slots = (uint8_t *)ctx->arena0 + scr_b;
    // results: records, then the packed blob (at most the slots' size)
    const size_t rb = al(sizeof(bsb_cigar_out_t) * (size_t)n);
    if ((rc = bsb_ensure(ctx, &ctx->d_out, &ctx->d_out_bytes, rb + slot_b, "CIGAR output"))) return rc;
    bsb_cigar_out_t *d_out = (bsb_cigar_out_t *)ctx->d_out;
    uint8_t *d_blob = (uint8_t *)ctx->d_out + rb;
    // one warp per job: as many blocks as are resident, or one per kCigarWarps jobs
    static int resident = 0;
    if (!resident) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, cigar_kernel, kCigarBlock, 0) != cudaSuccess || b < 1)
            b = 1;
        resident = b;
    }
    const int wblocks = (int)std::min<int64_t>(((int64_t)n + kCigarWarps - 1) / kCigarWarps,
                                               (int64_t)ctx->n_sm * resident);
    cigar_kernel<<<wblocks, kCigarBlock, 0, st>>>(P, d_jobs, n, (const uint8_t *)ctx->idx_pac,
                                                 (const uint8_t *)ctx->idx_opac, d_q, d_o, d_scr_off, d_slot_off,
                                                 d_scr, d_slots, d_out, d_bytes);
    if ((rc = bsb_cuda(ctx, scan_i32_i64(d_bytes, n, d_off, d_tmp, st), "CIGAR record offsets"))) return rc;
    // one warp per record: the copies are short and latency-bound
    const int cblocks = (int)std::min<int64_t>(((int64_t)n + kCigarWarps - 1) / kCigarWarps, 1 << 20);
    compact_kernel<<<cblocks, kCigarBlock, 0, st>>>(d_slots, d_slot_off, d_bytes, d_off, n, d_blob, d_out);
    if ((rc = bsb_cuda(ctx, cudaGetLastError(), "CIGAR kernels"))) return rc;
    int64_t used = 0;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(out, d_out, sizeof(bsb_cigar_out_t) * n, cudaMemcpyDeviceToHost, st),
                       "D2H records")) ||
        (rc = bsb_cuda(ctx, cudaMemcpyAsync(&used, d_off + n, 8, cudaMemcpyDeviceToHost, st), "D2H blob size")) ||
        (rc = bsb_cuda(ctx, cudaStreamSynchronize(st), "CIGAR batch")))
        return rc;
    *blob_used = used;
    if (used > blob_cap)
        return bsb_fail(ctx, BSB_EINVAL, "CIGAR records need %lld bytes, blob holds %lld", (long long)used,
                        (long long)blob_cap);
    if (used > 0 && (rc = bsb_cuda(ctx, cudaMemcpyAsync(blob, d_blob, used, cudaMemcpyDeviceToHost, st), "D2H blob")))
        return rc;
    return bsb_cuda(ctx, cudaStreamSynchronize(st), "CIGAR batch");
}
