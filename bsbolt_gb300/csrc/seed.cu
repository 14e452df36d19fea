// seed.cu -- SMEM seeding (mem_collect_intv) and suffix-array lookups on sm_103a.
//
// One thread carries one read through the three passes of mem_collect_intv
// (bsbolt/External/BWA/bwamem.c:118-166):
//   pass 1  bwt_smem1 from every x (bwt.c:289-356), keep SMEMs >= min_seed_len;
//   pass 2  re-seed from the middle of SMEMs >= split_len with <= split_width hits;
//   pass 3  bwt_seed_strategy1 (bwt.c:358-379) from every x.
// then sorts the read's seeds by info.  Equal info means the same substring
// and so the same interval, so the sort needs no tie rule.  The interval
// lists of bwt_smem1 live in a per-thread slice of device scratch (they are
// short in practice, but a repeat can make them as long as the read).
// Every occurrence query reads one or two 64-byte BWT blocks (fm_index.cuh).
//
// bwt_sa (bwt.c:86-96) is one thread per suffix-array row: LF steps until a
// sampled row, each step one 64-byte block.

#include "bsb_internal.cuh"
#include "fm_index.cuh"

namespace {

constexpr int kSeedBlock = 128;

struct SeedOpt {
    int min_seed_len, split_len, split_width, max_mem_intv;
};

// bwt_smem1 == bwt_smem1a(max_intv = 0).  mem receives the SMEMs covering x, sorted
// by start; returns the end of the longest match from x.  lists: 2*(len+2) entries.
__device__ int smem1(const DevFM &F, int len, const uint8_t *__restrict__ q, int x, int min_intv,
                     DevIntv *__restrict__ mem, int &n_mem, DevIntv *__restrict__ lists, int cap)
{
    DevIntv ik, ok[4];
    DevIntv *curr = lists, *prev = lists + cap;
    int i, n_curr = 0, n_prev, ret;
    n_mem = 0;
    if (q[x] > 3) return x + 1;
    if (min_intv < 1) min_intv = 1;
    ik = set_intv(F, q[x]);
    ik.info = (uint64_t)(x + 1);
    // forward: remember the interval whenever its size is about to change
    for (i = x + 1; i < len; ++i) {
        const int b = q[i];
        if (b < 4) {
            const int c = 3 - b;
            bwt_extend_dev(F, ik, ok, false);
            if (ok[c].x2 != ik.x2) {
                curr[n_curr++] = ik;
                if (ok[c].x2 < (uint64_t)min_intv) break;
            }
            ik = ok[c];
            ik.info = (uint64_t)(i + 1);
        } else {
            curr[n_curr++] = ik;
            break;
        }
    }
    if (i == len) curr[n_curr++] = ik;
    for (int j = 0; j < n_curr / 2; ++j) {
        DevIntv t = curr[j];
        curr[j] = curr[n_curr - 1 - j];
        curr[n_curr - 1 - j] = t;
    }
    ret = (int)(uint32_t)curr[0].info;
    { DevIntv *s = curr; curr = prev; prev = s; }
    n_prev = n_curr;
    // backward: grow every remembered interval to the left
    for (i = x - 1; i >= -1; --i) {
        const int c = i < 0 ? -1 : (q[i] < 4 ? q[i] : -1);
        n_curr = 0;
        for (int j = 0; j < n_prev; ++j) {
            const DevIntv p = prev[j];
            if (c >= 0) bwt_extend_dev(F, p, ok, true);
            if (c < 0 || ok[c].x2 < (uint64_t)min_intv) {
                if (n_curr == 0) {
                    if (n_mem == 0 || (uint64_t)(i + 1) < (mem[n_mem - 1].info >> 32)) {
                        DevIntv m = p;
                        m.info |= (uint64_t)(i + 1) << 32;
                        mem[n_mem++] = m;
                    }
                }
            } else if (n_curr == 0 || ok[c].x2 != curr[n_curr - 1].x2) {
                DevIntv m = ok[c];
                m.info = p.info;
                curr[n_curr++] = m;
            }
        }
        if (n_curr == 0) break;
        { DevIntv *s = curr; curr = prev; prev = s; }
        n_prev = n_curr;
    }
    for (int j = 0; j < n_mem / 2; ++j) {
        DevIntv t = mem[j];
        mem[j] = mem[n_mem - 1 - j];
        mem[n_mem - 1 - j] = t;
    }
    return ret;
}

__device__ int seed_strategy1(const DevFM &F, int len, const uint8_t *__restrict__ q, int x, int min_len,
                              int max_intv, DevIntv &mem)
{
    DevIntv ik, ok[4];
    mem.x0 = mem.x1 = mem.x2 = mem.info = 0;
    if (q[x] > 3) return x + 1;
    ik = set_intv(F, q[x]);
    for (int i = x + 1; i < len; ++i) {
        if (q[i] < 4) {
            const int c = 3 - q[i];
            bwt_extend_dev(F, ik, ok, false);
            if (ok[c].x2 < (uint64_t)max_intv && i - x >= min_len) {
                mem = ok[c];
                mem.info = (uint64_t)x << 32 | (uint64_t)(i + 1);
                return i + 1;
            }
            ik = ok[c];
        } else return i + 1;
    }
    return len;
}

__device__ __forceinline__ int seed_len(const DevIntv &p)
{
    return (int)((uint32_t)p.info - (uint32_t)(p.info >> 32));
}

// Persistent: each thread takes reads from a counter.  out holds, per read r,
// cap(r) = 2*len(r) + 32 slots starting at 2*(offs[r]-offs[0]) + 32*r.
__global__ void __launch_bounds__(kSeedBlock)
seed_kernel(DevFM F, SeedOpt opt, int n_reads, const uint8_t *__restrict__ seqs, const int64_t *__restrict__ offs,
            DevIntv *__restrict__ out, int *__restrict__ count, DevIntv *__restrict__ scratch, int list_cap,
            int *__restrict__ next_read, int *__restrict__ overflow)
{
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    DevIntv *lists = scratch + (size_t)tid * 3 * list_cap;   // curr/prev lists, then mem
    DevIntv *mem = lists + 2 * list_cap;
    const int64_t base_off = offs[0];
    for (;;) {
        const int r = atomicAdd(next_read, 1);
        if (r >= n_reads) break;
        const int64_t o = offs[r];
        const int64_t len64 = offs[r + 1] - o;
        if (len64 < 0 || len64 > list_cap - 2) {    // outside the scratch the launch sized: refuse, never overrun
            count[r] = 0;
            atomicMax(overflow, r + 1);
            continue;
        }
        const int len = (int)len64;
        const uint8_t *q = seqs + o;
        DevIntv *dst = out + 2 * (o - base_off) + 32 * (int64_t)r;
        const int cap = 2 * len + 32;
        int n = 0, nm;
        if (len < opt.min_seed_len) {     // mem_chain returns before seeding (bwamem.c:266)
            count[r] = 0;
            continue;
        }
        // pass 1
        for (int x = 0; x < len;) {
            if (q[x] < 4) {
                x = smem1(F, len, q, x, 1, mem, nm, lists, list_cap);
                for (int i = 0; i < nm; ++i)
                    if (seed_len(mem[i]) >= opt.min_seed_len) {
                        if (n < cap) dst[n] = mem[i];
                        ++n;
                    }
            } else ++x;
        }
        // pass 2
        const int old_n = n < cap ? n : cap;
        for (int k = 0; k < old_n; ++k) {
            const DevIntv p = dst[k];
            const int start = (int)(p.info >> 32), end = (int)(uint32_t)p.info;
            if (end - start < opt.split_len || p.x2 > (uint64_t)opt.split_width) continue;
            smem1(F, len, q, (start + end) >> 1, (int)p.x2 + 1, mem, nm, lists, list_cap);
            for (int i = 0; i < nm; ++i)
                if (seed_len(mem[i]) >= opt.min_seed_len) {
                    if (n < cap) dst[n] = mem[i];
                    ++n;
                }
        }
        // pass 3
        if (opt.max_mem_intv > 0) {
            for (int x = 0; x < len;) {
                if (q[x] < 4) {
                    DevIntv m;
                    x = seed_strategy1(F, len, q, x, opt.min_seed_len, opt.max_mem_intv, m);
                    if (m.x2 > 0) {
                        if (n < cap) dst[n] = m;
                        ++n;
                    }
                } else ++x;
            }
        }
        if (n > cap) {
            atomicMax(overflow, r + 1);
            n = cap;
        }
        // insertion sort by info (ks_introsort with intv_lt, bwamem.c:92-93; equal keys are equal values)
        for (int i = 1; i < n; ++i) {
            const DevIntv v = dst[i];
            int j = i - 1;
            while (j >= 0 && dst[j].info > v.info) {
                dst[j + 1] = dst[j];
                --j;
            }
            dst[j + 1] = v;
        }
        count[r] = n;
    }
}

// Exclusive scan of per-read counts into out_off[0..n] (single block, chunked).
__global__ void scan_counts(const int *__restrict__ count, int n, int64_t *__restrict__ out_off)
{
    __shared__ int64_t part[1024];
    const int t = threadIdx.x, T = blockDim.x;
    const int per = (n + T - 1) / T;
    const int lo = t * per, hi = min(n, lo + per);
    int64_t s = 0;
    for (int i = lo; i < hi; ++i) s += count[i];
    part[t] = s;
    __syncthreads();
    if (t == 0) {
        int64_t acc = 0;
        for (int i = 0; i < T; ++i) {
            const int64_t v = part[i];
            part[i] = acc;
            acc += v;
        }
        out_off[n] = acc;
    }
    __syncthreads();
    int64_t acc = part[t];
    for (int i = lo; i < hi; ++i) {
        out_off[i] = acc;
        acc += count[i];
    }
}

__global__ void compact_seeds(const DevIntv *__restrict__ padded, const int64_t *__restrict__ offs, int n_reads,
                              const int *__restrict__ count, const int64_t *__restrict__ out_off,
                              DevIntv *__restrict__ out)
{
    const int64_t base_off = offs[0];
    for (int r = blockIdx.x; r < n_reads; r += gridDim.x) {
        const DevIntv *src = padded + 2 * (offs[r] - base_off) + 32 * (int64_t)r;
        DevIntv *dst = out + out_off[r];
        for (int i = threadIdx.x; i < count[r]; i += blockDim.x) dst[i] = src[i];
    }
}

// bwt_sa: LF-walk to the nearest sampled row (bwt.c:53-59, 86-96).
// Rows beyond seq_len are answered with (uint64_t)-2 and never walked.
__global__ void sa_kernel(DevFM F, const uint64_t *__restrict__ rows, int64_t n, uint64_t *__restrict__ pos)
{
    const uint64_t mask = (1ull << F.sa_shift) - 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t k = rows[i], steps = 0;
        if (k > F.seq_len) {
            pos[i] = ~(uint64_t)1;
            continue;
        }
        while (k & mask) {
            ++steps;
            if (k == F.primary) {
                k = 0;
                continue;
            }
            const uint64_t kk = k - (k >= F.primary);
            const Block b = load_block(F, kk);
            const uint64_t xs = k - (k > F.primary);    // symbol row (bwt_invPsi uses >, bwt.c:55)
            const int c = (int)(block_word(b, (int)((xs & 127) >> 4)) >> ((~xs & 15) << 1) & 3);
            // xs and kk differ only when k == primary, handled above, so one block serves both
            const Occ4 o = occ_in_block(b, kk);
            k = F.L2[c] + o.c[c];
        }
        pos[i] = steps + __ldg(F.sa + (k >> F.sa_shift));
    }
}

}  // namespace

size_t seed_scratch_bytes(int n_threads, int max_len)
{
    return (size_t)n_threads * 3 * (size_t)(max_len + 2) * sizeof(DevIntv);
}

// Persistent seeding threads: 4 blocks per SM, fewer when long reads would make
// the per-thread interval lists exceed ~1 GB of scratch.
int seed_threads(int n_sm, int max_len)
{
    const size_t per_block = (size_t)kSeedBlock * 3 * (size_t)(max_len + 2) * sizeof(DevIntv);
    size_t blocks = (size_t)n_sm * 4;
    const size_t budget = (size_t)1 << 30;
    if (blocks * per_block > budget) blocks = budget / per_block;
    if (blocks < (size_t)n_sm) blocks = n_sm;
    return (int)blocks * kSeedBlock;
}

size_t seed_padded_entries(int64_t total_bases, int n_reads)
{
    return 2 * (size_t)total_bases + 32 * (size_t)n_reads;
}

cudaError_t seed_launch(const DevFM &F, int min_seed_len, float split_factor, int split_width, int max_mem_intv,
                        int n_reads, const uint8_t *d_seqs, const int64_t *d_offs, int max_len,
                        void *d_padded, int *d_count, int64_t *d_out_off, void *d_out,
                        void *d_lists, int *d_ctrl, int n_sm, cudaStream_t st)
{
    SeedOpt o;
    o.min_seed_len = min_seed_len;
    o.split_len = (int)(min_seed_len * split_factor + .499);    // bwamem.c:122
    o.split_width = split_width;
    o.max_mem_intv = max_mem_intv;
    cudaError_t e = cudaMemsetAsync(d_ctrl, 0, 2 * sizeof(int), st);
    if (e != cudaSuccess) return e;
    const int blocks = seed_threads(n_sm, max_len) / kSeedBlock;
    seed_kernel<<<blocks, kSeedBlock, 0, st>>>(F, o, n_reads, d_seqs, d_offs, (DevIntv *)d_padded, d_count,
                                               (DevIntv *)d_lists, max_len + 2, d_ctrl, d_ctrl + 1);
    scan_counts<<<1, 1024, 0, st>>>(d_count, n_reads, d_out_off);
    compact_seeds<<<n_sm * 4, 128, 0, st>>>((const DevIntv *)d_padded, d_offs, n_reads, d_count, d_out_off,
                                            (DevIntv *)d_out);
    return cudaGetLastError();
}

cudaError_t sa_launch(const DevFM &F, const uint64_t *d_rows, int64_t n, uint64_t *d_pos, int n_sm, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const int64_t want = (n + 255) / 256;
    const int blocks = (int)(want < (int64_t)n_sm * 16 ? want : (int64_t)n_sm * 16);
    sa_kernel<<<blocks, 256, 0, st>>>(F, d_rows, n, d_pos);
    return cudaGetLastError();
}
