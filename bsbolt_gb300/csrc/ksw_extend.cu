// ksw_extend.cu -- batched ksw_extend2 for sm_103a.
//
// Bit-exact restatement of the reference banded extension
// (bsbolt/External/BWA/ksw.c:380-479) as one warp per job.
//
// Why row-parallel and not an anti-diagonal wavefront: the reference decides
// each row's band [beg,end) from the complete previous row (the shrink to
// non-zero cells, ksw.c:466-469), stops on a zero row (ksw.c:454) and tests
// z-drop per target row (ksw.c:458-464).  A wavefront would have to run rows
// whose band is not known yet.  Instead the warp computes a whole row at once:
//   * lane L owns query columns [L*C, L*C+C) in registers (C = tile width,
//     a template parameter, picked per job from qlen);
//   * M and E depend only on the previous row and are computed per cell;
//   * F(i,j+1) = max(F(i,j) - e_ins, max(M(i,j) - oe_ins, 0)) is a max-plus
//     recurrence along the row, solved exactly with a warp prefix-max scan of
//     T(k) + e_ins*(k+1) (one __shfl_up_sync ladder per row);
//   * the row maximum, its last column, and the first/last non-zero cell of
//     the shrink are warp reductions (redux.sync).
// The register file holds the reference's whole eh[] array, including cells
// outside the current band: the band may grow back over them and read stale
// values, exactly as the reference does.
//
// Scheduling (the plain schedule): jobs are binned by tile width C and, within
// a bin, issued longest-bound-first (qlen x min(tlen, qlen+w), or a caller
// supplied cost key); each bin runs as a persistent kernel whose warps pull
// jobs from a device counter.  Results never depend on the order.

#include <climits>
#include <cstdio>

#include "bsb_internal.cuh"

namespace {

// Tile widths (query columns per lane).  C covers qlen <= 32*C - 1.
constexpr int kTiles[] = {1, 2, 3, 4, 5, 6, 7, 8, 10, 12, 16, 24, 32};
constexpr int kNumBins = sizeof(kTiles) / sizeof(kTiles[0]);
constexpr int kClasses = 128;           // cost classes within a bin
constexpr int kBlock = 128;             // threads per block (4 warps)

// Bin of the smallest tile in kTiles that holds columns 0..qlen.
__host__ __device__ inline int tile_bin(int qlen)
{
    const int need = (qlen + 32) >> 5;
    if (need <= 8) return need - 1;
    if (need <= 10) return 8;
    if (need <= 12) return 9;
    if (need <= 16) return 10;
    if (need <= 24) return 11;
    if (need <= 32) return 12;
    return -1;
}

// Sign-extended byte of x chosen by a prmt selector (bit 3 of each selector
// nibble replicates the sign of the chosen byte, PTX ISA prmt.b32 default mode).
__device__ __forceinline__ int prmt_sext(uint32_t x, uint32_t sel)
{
    uint32_t r;
    asm("prmt.b32 %0, %1, 0, %2;" : "=r"(r) : "r"(x), "r"(sel));
    return (int)r;
}

__device__ __forceinline__ uint32_t sext_selector(int byte)
{
    const uint32_t b = (uint32_t)byte, r = b | 8u;
    return b | r << 4 | r << 8 | r << 12;
}

// Extends one job with the calling warp.  All control values are warp-uniform.
//
// Register state per lane, columns j = lane*C + s:
//   Hs[s] = eh[j].h = H(i-1, j-1),  Es[s] = eh[j].e = E(i, j)   (ksw.c:376-378)
// Invariant: every column left of the band (j < beg) holds H = E = 0.  The
// reference never reads those cells again (beg only grows), and with them at
// zero the F scan and the row maximum need no left-edge masks: a dead column
// has M = 0, T = 0, V = e_ins*(j+1), F = 0 and H = 0.  The shrink step only
// moves beg over cells that are already zero; when the band edge i-w moves
// beg instead, the cells it passes are zeroed explicitly.
template <int C>
__device__ __forceinline__ void ksw_one(const KswParams &P, const bsb_ext_job_t &jb,
                                        const uint8_t *__restrict__ seq, int lane,
                                        bsb_ext_out_t *__restrict__ o, int64_t *__restrict__ cell_out)
{
    const int qlen = jb.qlen, tlen = jb.tlen, h0 = jb.h0;
    const uint8_t *__restrict__ q = seq + jb.qoff;
    const uint8_t *__restrict__ t = seq + jb.toff;
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
        const int qc = j < qlen ? q[j] : 0;
        prof[s] = (uint32_t)(uint8_t)P.mat[qc] | (uint32_t)(uint8_t)P.mat[5 + qc] << 8 |
                  (uint32_t)(uint8_t)P.mat[10 + qc] << 16 | (uint32_t)(uint8_t)P.mat[15 + qc] << 24;
        profN[s >> 2] |= (uint32_t)(uint8_t)P.mat[20 + qc] << ((s & 3) * 8);
        // first row: h0, then an insertion run clipped at zero (ksw.c:395-397)
        Hs[s] = j == 0 ? h0 : (j <= qlen ? max(h1run - e_ins * (j - 1), 0) : 0);
        Es[s] = 0;
    }

    // band clamp with the reference's double arithmetic (ksw.c:399-407)
    int w = jb.w;
    {
        int max_ins = (int)((double)(qlen * P.mat_max + jb.end_bonus - o_ins) / e_ins + 1.);
        max_ins = max_ins > 1 ? max_ins : 1;
        w = w < max_ins ? w : max_ins;
        int max_del = (int)((double)(qlen * P.mat_max + jb.end_bonus - o_del) / e_del + 1.);
        max_del = max_del > 1 ? max_del : 1;
        w = w < max_del ? w : max_del;
    }

    int best = h0, best_i = -1, best_j = -1, max_ie = -1, gscore = -1, max_off = 0;
    int beg = 0, end = qlen;
    long long ncell = 0;
    const int q_lane = qlen / C, q_slot = qlen % C;   // owner of column qlen

    // target bases arrive 32 rows at a time, one byte per lane, next chunk prefetched
    uint32_t tch = lane < tlen ? t[lane] : 4u;
    uint32_t tnext = 32 + lane < tlen ? t[32 + lane] : 4u;

    for (int i = 0; i < tlen; ++i) {
        const int tc = (int)__shfl_sync(BSB_FULL_MASK, tch, i & 31);
        if ((i & 31) == 31) {
            tch = tnext;
            const int ti = i + 33 + lane;
            tnext = ti < tlen ? t[ti] : 4u;
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
            const int nE = lt ? En[s] : (j == end ? 0 : Es[s]);
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
    if (lane == 0) {
        bsb_ext_out_t r;
        r.score = best; r.qle = best_j + 1; r.tle = best_i + 1;
        r.gtle = max_ie + 1; r.gscore = gscore; r.max_off = max_off;
        *o = r;
        if (cell_out) *cell_out = ncell;
    }
}

// Persistent per-bin kernel: warps pull job indices from counter[bin].
template <int C>
__global__ void __launch_bounds__(kBlock)
ksw_bin_kernel(KswParams P, const bsb_ext_job_t *__restrict__ jobs, const uint8_t *__restrict__ seq,
               const int32_t *__restrict__ order, const int32_t *__restrict__ bin_start, int bin,
               int *__restrict__ counter, bsb_ext_out_t *__restrict__ out, int64_t *__restrict__ cells)
{
    const int lane = threadIdx.x & 31;
    const int lo = bin_start[bin], hi = bin_start[bin + 1];
    for (;;) {
        int idx = 0;
        if (lane == 0) idx = atomicAdd(counter + bin, 1);
        idx = __shfl_sync(BSB_FULL_MASK, idx, 0) + lo;
        if (idx >= hi) break;
        const int job = order[idx];
        const bsb_ext_job_t jb = jobs[job];
        ksw_one<C>(P, jb, seq, lane, out + job, cells ? cells + job : nullptr);
    }
}

__device__ __forceinline__ int cost_class(uint32_t key)
{
    // 4 classes per power of two; class 0 = cheapest
    if (key == 0) return 0;
    const int msb = 31 - __clz(key);
    const int frac = msb >= 2 ? (int)((key >> (msb - 2)) & 3) : (int)((key << (2 - msb)) & 3);
    const int c = msb * 4 + frac;
    return c < kClasses ? c : kClasses - 1;
}

// Histogram of (bin, class) keys.  Bins are major; within a bin, classes are
// laid out most expensive first so an ascending scan issues longest-first.
// A job that fails the preconditions (the host entry checks them; the device
// entry cannot) gets the reject key kRejectKey: it is counted, never issued,
// and its output is left untouched.
constexpr int kRejectKey = kNumBins * kClasses;
constexpr int kHistSlots = kNumBins * kClasses + 1;

__global__ void ksw_sched_hist(const bsb_ext_job_t *__restrict__ jobs, int n, long long seq_bytes,
                               const int32_t *__restrict__ cost, int *__restrict__ hist,
                               int32_t *__restrict__ key_out)
{
    __shared__ int sh[kHistSlots];
    for (int i = threadIdx.x; i < kHistSlots; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const bsb_ext_job_t jb = jobs[i];
        const int b = tile_bin(jb.qlen);
        const bool ok = b >= 0 && jb.qlen >= 0 && jb.tlen >= 0 && jb.w >= 0 && jb.h0 > 0 &&
                        jb.h0 <= (1 << 20) && jb.flags == 0 && jb.qoff >= 0 && jb.toff >= 0 &&
                        jb.qoff + jb.qlen <= seq_bytes && jb.toff + jb.tlen <= seq_bytes;
        int key;
        if (!ok) {
            key = kRejectKey;
        } else {
            uint32_t k;
            if (cost) k = (uint32_t)max(cost[i], 0);
            else {
                const long long span = min((long long)jb.tlen, (long long)jb.qlen + jb.w);
                const long long c = (long long)jb.qlen * max(span, 0LL);
                k = (uint32_t)min(c, (long long)0x7fffffff);
            }
            key = b * kClasses + (kClasses - 1 - cost_class(k));
        }
        key_out[i] = key;
        atomicAdd(&sh[key], 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kHistSlots; i += blockDim.x)
        if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// Exclusive scan of the histogram (single block) -> cursors and bin starts.
// bin_start[kNumBins] is where the rejected jobs begin; rejected[0] counts them.
__global__ void ksw_sched_scan(const int *__restrict__ hist, int *__restrict__ cursor,
                               int32_t *__restrict__ bin_start, int *__restrict__ rejected)
{
    __shared__ int s[kHistSlots];
    for (int i = threadIdx.x; i < kHistSlots; i += blockDim.x) s[i] = hist[i];
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int i = 0; i < kHistSlots; ++i) {
            const int v = s[i];
            s[i] = acc;
            acc += v;
        }
        for (int b = 0; b < kNumBins; ++b) bin_start[b] = s[b * kClasses];
        bin_start[kNumBins] = s[kRejectKey];
        rejected[0] = acc - s[kRejectKey];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kHistSlots; i += blockDim.x) cursor[i] = s[i];
}

__global__ void ksw_sched_scatter(const int32_t *__restrict__ key, int n, int *__restrict__ cursor,
                                  int32_t *__restrict__ order)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int pos = atomicAdd(&cursor[key[i]], 1);
        order[pos] = i;
    }
}

template <int C>
cudaError_t launch_bin(const KswParams &P, const bsb_ext_job_t *jobs, const uint8_t *seq,
                       const int32_t *order, const int32_t *bin_start, int bin, int *counter,
                       bsb_ext_out_t *out, int64_t *cells, int n_sm, cudaStream_t st)
{
    static int blocks_per_sm = 0;
    if (!blocks_per_sm) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, ksw_bin_kernel<C>, kBlock, 0);
        if (e != cudaSuccess) return e;
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    ksw_bin_kernel<C><<<n_sm * blocks_per_sm, kBlock, 0, st>>>(P, jobs, seq, order, bin_start, bin, counter, out, cells);
    return cudaGetLastError();
}

template <int I>
cudaError_t launch_all_bins(const KswParams &P, const bsb_ext_job_t *jobs, const uint8_t *seq,
                            const int32_t *order, const int32_t *bin_start, int *counter,
                            bsb_ext_out_t *out, int64_t *cells, int n_sm, cudaStream_t st)
{
    if constexpr (I == kNumBins) {
        return cudaSuccess;
    } else {
        cudaError_t e = launch_bin<kTiles[I]>(P, jobs, seq, order, bin_start, I, counter, out, cells, n_sm, st);
        if (e != cudaSuccess) return e;
        return launch_all_bins<I + 1>(P, jobs, seq, order, bin_start, counter, out, cells, n_sm, st);
    }
}

}  // namespace

// scratch layout (int32 words): counter[kNumBins] | rejected[1] | hist[kHistSlots] |
//   cursor[kHistSlots] | bin_start[kNumBins+1] | (256-byte aligned) key[n] | order[n]
static size_t fixed_bytes()
{
    size_t fixed = sizeof(int) * (kNumBins + 1 + 2 * kHistSlots + kNumBins + 1);
    return (fixed + 255) & ~(size_t)255;
}

size_t ksw_scratch_bytes(int64_t n) { return fixed_bytes() + sizeof(int32_t) * 2 * (size_t)n + 256; }

int ksw_max_qlen() { return 32 * kTiles[kNumBins - 1] - 1; }

int *ksw_rejected_counter(void *scratch) { return (int *)scratch + kNumBins; }

cudaError_t ksw_launch(const KswParams &P, const bsb_ext_job_t *d_jobs, int64_t n, int64_t seq_bytes,
                       const uint8_t *d_seq, const int32_t *d_cost, bsb_ext_out_t *d_out,
                       int64_t *d_cells, void *scratch, int n_sm, cudaStream_t st,
                       cudaEvent_t ev0, cudaEvent_t ev1)
{
    char *p = (char *)scratch;
    int *counter = (int *)p;
    int *rejected = counter + kNumBins;
    int *hist = rejected + 1;
    int *cursor = hist + kHistSlots;
    int32_t *bin_start = cursor + kHistSlots;
    int32_t *key = (int32_t *)(p + fixed_bytes());
    int32_t *order = key + n;
    cudaError_t e;
    if (ev0) cudaEventRecord(ev0, st);
    e = cudaMemsetAsync(scratch, 0, sizeof(int) * (kNumBins + 1 + kHistSlots), st);
    if (e != cudaSuccess) return e;
    if (n > 0) {
        const int nb = (int)min((int64_t)n_sm * 8, (n + 255) / 256);
        ksw_sched_hist<<<nb, 256, 0, st>>>(d_jobs, (int)n, (long long)seq_bytes, d_cost, hist, key);
        ksw_sched_scan<<<1, 256, 0, st>>>(hist, cursor, bin_start, rejected);
        ksw_sched_scatter<<<nb, 256, 0, st>>>(key, (int)n, cursor, order);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        e = launch_all_bins<0>(P, d_jobs, d_seq, order, bin_start, counter, d_out, d_cells, n_sm, st);
        if (e != cudaSuccess) return e;
    }
    if (ev1) cudaEventRecord(ev1, st);
    return cudaSuccess;
}
