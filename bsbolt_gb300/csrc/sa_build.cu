// sa_build.cu -- the suffixes of BWA's index text, sorted on the GPU.
//
// bwa index sorts the suffixes of the forward 2-bit pac followed by its reverse complement
// (2*l_pac symbols, bntseq.c / bwtindex.c) with a sentinel '$' that sorts before every base;
// the BWT, the occurrence array and the sampled SA (.bwt, .sa) are read off that order.
// On the host (host_index.c) an SA-IS with 32-bit indexes does this up to 2^31 symbols and
// takes minutes per billion.  Here prefix doubling runs on device radix sorts (CUB, part of
// the CUDA toolkit): every suffix is first keyed by its next 21 symbols (3 bits each, 0 past
// the end) and sorted; then each round keys suffix i by (rank[i], rank[i + h]) and sorts again,
// h = 21, 42, 84, ... until every rank is distinct.  Suffixes whose first h symbols reach the
// sentinel are already alone in their group, so rank[i + h] past the end can be anything.
//   bsb_build_suffix_array: 32-bit ranks (texts below 2^32 - 1 symbols), all suffixes sorted
//   together each round, the whole array copied back (~33 bytes of device memory per symbol).
//   bsb_build_bwt: 64-bit ranks, suffixes sorted in chunks that fit device memory, only the
//   BWT and the sampled rows copied back (described above the function).

#include <algorithm>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "bsb_internal.cuh"

namespace {

constexpr int kPrefixSyms = 21;          // 21 symbols x 3 bits in the first 63-bit key

// text[p] for p < n: the pac base at p, then the reverse complement of the pac.
__global__ void text_kernel(const uint8_t *__restrict__ pac, int64_t l_pac, uint8_t *__restrict__ text)
{
    const int64_t n = 2 * l_pac;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = p < l_pac ? p : 2 * l_pac - 1 - p;
        const int b = pac[q >> 2] >> ((~q & 3) << 1) & 3;
        text[p] = (uint8_t)(p < l_pac ? b : 3 - b);
    }
}

// key of suffix i: its next 21 symbols, code + 1 each, 0 past the end (the sentinel sorts first).
__global__ void first_keys(const uint8_t *__restrict__ text, int64_t n, uint64_t *__restrict__ key,
                           uint32_t *__restrict__ idx)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t k = 0;
        for (int j = 0; j < kPrefixSyms; ++j) {
            const int64_t p = i + j;
            k = k << 3 | (p < n ? (uint64_t)text[p] + 1 : 0);
        }
        key[i] = k;
        idx[i] = (uint32_t)i;
    }
}

// Row j of the sorted order starts a group when its key differs from row j-1's: head[j] = j,
// else 0; an inclusive max-scan of head then gives every row its group's first row.
__global__ void group_heads(const uint64_t *__restrict__ key, int64_t m, uint32_t *__restrict__ head)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x)
        head[j] = (j == 0 || key[j] != key[j - 1]) ? (uint32_t)j : 0u;
}

__global__ void count_heads(const uint64_t *__restrict__ key, int64_t m, unsigned long long *__restrict__ groups)
{
    unsigned c = 0;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x)
        c += (j == 0 || key[j] != key[j - 1]);
    c = __reduce_add_sync(BSB_FULL_MASK, c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(groups, (unsigned long long)c);
}

__global__ void scatter_rank(const uint32_t *__restrict__ idx, const uint32_t *__restrict__ grp, int64_t m,
                             uint32_t *__restrict__ rank)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x)
        rank[idx[j]] = grp[j];
}

// The next round's key of the suffix at sorted row j: (rank[i], rank[i + h]).
__global__ void pair_keys(const uint32_t *__restrict__ idx, const uint32_t *__restrict__ rank, int64_t m, int64_t h,
                          uint64_t *__restrict__ key)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx[j];
        const uint32_t r2 = i + h < m ? rank[i + h] : 0u;
        key[j] = (uint64_t)rank[i] << 32 | r2;
    }
}

__global__ void widen_rows(const uint32_t *__restrict__ idx, int64_t m, uint64_t *__restrict__ out)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x)
        out[j] = idx[j];
}

struct DevBuf {                          // freed on every return (after the stream is idle or failed)
    void *p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
};

}  // namespace

extern "C" int bsb_build_suffix_array(bsb_ctx *ctx, const uint8_t *pac, int64_t l_pac, int64_t *sa)
{
    if (!ctx) return BSB_EINVAL;
    if (!pac || !sa || l_pac < 1) return bsb_fail(ctx, BSB_EINVAL, "NULL argument or empty pac");
    const int64_t n = 2 * l_pac, m = n + 1;      // suffixes 0..n, n = the sentinel
    if (m > (int64_t)0xffffffffLL)
        return bsb_fail(ctx, BSB_ETOOLONG, "text of %lld symbols: ranks are 32-bit", (long long)n);
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    cudaStream_t st = ctx->stream;
    const size_t pb = (size_t)(l_pac + 3) / 4;
    DevBuf d_pac, d_text, k0, k1, v0, v1, d_rank, d_tmp, d_cnt;
    size_t tmp_sort = 0, tmp_scan = 0;
    cub::DoubleBuffer<uint64_t> keys;
    cub::DoubleBuffer<uint32_t> vals;
    if (cub::DeviceRadixSort::SortPairs(nullptr, tmp_sort, keys, vals, m, 0, 64, st) != cudaSuccess ||
        cub::DeviceScan::InclusiveScan(nullptr, tmp_scan, (uint32_t *)nullptr, (uint32_t *)nullptr, cuda::maximum<>(),
                                       m, st) != cudaSuccess)
        return bsb_fail(ctx, BSB_ECUDA, "suffix array: sort set-up");
    const size_t tmp_bytes = tmp_sort > tmp_scan ? tmp_sort : tmp_scan;
    if ((rc = bsb_cuda(ctx, cudaMalloc(&d_pac.p, pb + 16), "suffix array: pac")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&d_text.p, (size_t)n + 16), "suffix array: text")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&k0.p, 8 * (size_t)m), "suffix array: keys")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&k1.p, 8 * (size_t)m), "suffix array: keys")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&v0.p, 4 * (size_t)m), "suffix array: rows")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&v1.p, 4 * (size_t)m), "suffix array: rows")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&d_rank.p, 4 * (size_t)m), "suffix array: ranks")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&d_tmp.p, tmp_bytes + 256), "suffix array: sort scratch")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&d_cnt.p, 64), "suffix array: counter")))
        return rc;
    const int grid = ctx->n_sm * 16;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(d_pac.p, pac, pb, cudaMemcpyHostToDevice, st), "suffix array: H2D pac")))
        return rc;
    text_kernel<<<grid, 256, 0, st>>>((const uint8_t *)d_pac.p, l_pac, (uint8_t *)d_text.p);
    keys = cub::DoubleBuffer<uint64_t>((uint64_t *)k0.p, (uint64_t *)k1.p);
    vals = cub::DoubleBuffer<uint32_t>((uint32_t *)v0.p, (uint32_t *)v1.p);
    first_keys<<<grid, 256, 0, st>>>((const uint8_t *)d_text.p, n, keys.Current(), vals.Current());
    unsigned long long groups = 0;
    for (int64_t h = kPrefixSyms, round = 0;; h *= 2, ++round) {
        size_t t = tmp_bytes;
        if ((rc = bsb_cuda(ctx, cub::DeviceRadixSort::SortPairs(d_tmp.p, t, keys, vals, m, 0, 64, st), "suffix sort")))
            return rc;
        if ((rc = bsb_cuda(ctx, cudaMemsetAsync(d_cnt.p, 0, 8, st), "suffix array: counter"))) return rc;
        count_heads<<<grid, 256, 0, st>>>(keys.Current(), m, (unsigned long long *)d_cnt.p);
        if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(&groups, d_cnt.p, 8, cudaMemcpyDeviceToHost, st), "D2H groups")) ||
            (rc = bsb_cuda(ctx, cudaStreamSynchronize(st), "suffix array round")))
            return rc;
        if ((int64_t)groups == m) break;            // every suffix has its own rank: done
        if (round > 40) return bsb_fail(ctx, BSB_EINVAL, "suffix array: no convergence");
        // group first rows into the spare index buffer, then ranks by suffix
        uint32_t *head = vals.Alternate();
        group_heads<<<grid, 256, 0, st>>>(keys.Current(), m, head);
        t = tmp_bytes;
        if ((rc = bsb_cuda(ctx, cub::DeviceScan::InclusiveScan(d_tmp.p, t, head, head, cuda::maximum<>(), m, st),
                           "suffix array: group scan")))
            return rc;
        scatter_rank<<<grid, 256, 0, st>>>(vals.Current(), head, m, (uint32_t *)d_rank.p);
        pair_keys<<<grid, 256, 0, st>>>(vals.Current(), (const uint32_t *)d_rank.p, m, h, keys.Current());
    }
    // the order of the suffixes, as int64, through the spare key buffer
    uint64_t *out = keys.Alternate();
    widen_rows<<<grid, 256, 0, st>>>(vals.Current(), m, out);
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(sa, out, 8 * (size_t)m, cudaMemcpyDeviceToHost, st), "D2H suffix array")))
        return rc;
    return bsb_cuda(ctx, cudaStreamSynchronize(st), "suffix array");
}

// ---------------------------------------------------------------- BWT and sampled SA, any length
//
// bsb_build_bwt sorts the same suffixes without a 32-bit limit and returns what bwa index writes
// from the order -- the BWT (2-bit symbols, 16 per word, the row of suffix 0 left out) and every
// sa_intv-th row of the suffix array -- instead of the whole array.  Device memory is the text
// (1 byte per symbol), a 64-bit rank per suffix, and the buffers of one sort: suffixes are sorted
// in chunks that fit the memory left over.
//   Round 0: suffixes are bucketed by their first 5 symbols (codes 0..4, 0 past the end, as a
//   base-5 number, which keeps the key order); a chunk is a run of whole buckets, gathered, sorted
//   by the 21-symbol key, and every suffix gets the sorted position of its group's last row as
//   its rank (the chunk's first position is the count of the buckets before it).
//   Round r: the suffixes not yet alone in their group (bit 63 of the rank clear) are binned by
//   rank; a chunk is a run of whole bins (so of whole groups), keyed by (rank[i] - chunk's first
//   rank, rank[i + h]) in one 64-bit key, sorted, and given last-row ranks again.  Ranks are
//   written back chunk by chunk, so later chunks of a round may read ranks of i + h that are
//   already finer than h symbols; they are still consistent with the suffix order, and sorting by
//   them refines each group at least to 2h symbols (Larsson and Sadakane's qsufsort argument).
//   A refined group's ranks only move down, into bins an earlier chunk of the round has already
//   taken, so every chunk gathers exactly the suffixes its bins counted.  A suffix shorter than
//   h symbols is alone in its group after the round of h, so i + h <= n for every suffix still
//   to be sorted.
//   Last: rank[i] is suffix i's row; BWT[row] = text[i - 1] and SA[row] = i for sampled rows.

namespace {

constexpr uint64_t kAlone = 1ull << 63;     // rank flag: the suffix's group has one member
constexpr int kBucketSyms = 5, kBuckets = 3125;    // 5^5 buckets of round 0
constexpr int kBinBits = 13;                 // rounds >= 1: up to 2^13 rank bins

__device__ __forceinline__ uint32_t code_at(const uint8_t *__restrict__ text, int64_t n, int64_t p)
{
    return p < n ? (uint32_t)text[p] + 1u : 0u;
}

__device__ __forceinline__ int bucket_of(const uint8_t *__restrict__ text, int64_t n, int64_t i)
{
    int b = 0;
#pragma unroll
    for (int j = 0; j < kBucketSyms; ++j) b = b * 5 + (int)code_at(text, n, i + j);
    return b;
}

__device__ __forceinline__ uint64_t key21(const uint8_t *__restrict__ text, int64_t n, int64_t i)
{
    uint64_t k = 0;
#pragma unroll
    for (int j = 0; j < kPrefixSyms; ++j) k = k << 3 | code_at(text, n, i + j);
    return k;
}

// per-block histogram in shared memory, added to the global bins
__global__ void bucket_hist(const uint8_t *__restrict__ text, int64_t n, unsigned long long *__restrict__ hist)
{
    __shared__ unsigned sh[kBuckets];
    for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) sh[b] = 0;
    __syncthreads();
    const int64_t m = n + 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&sh[bucket_of(text, n, i)], 1u);
    __syncthreads();
    for (int b = threadIdx.x; b < kBuckets; b += blockDim.x)
        if (sh[b]) atomicAdd(&hist[b], (unsigned long long)sh[b]);
}

__global__ void rank_hist(const uint64_t *__restrict__ rank, int64_t m, int shift, int n_bins,
                          unsigned long long *__restrict__ hist)
{
    __shared__ unsigned sh[1 << kBinBits];
    for (int b = threadIdx.x; b < n_bins; b += blockDim.x) sh[b] = 0;
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t r = rank[i];
        if (!(r & kAlone)) atomicAdd(&sh[(int)(r >> shift)], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < n_bins; b += blockDim.x)
        if (sh[b]) atomicAdd(&hist[b], (unsigned long long)sh[b]);
}

// Appends (key, i) for the selected suffixes at a warp-aggregated slot; every lane of a warp runs
// the same iterations (the ballot is over the full warp).
__device__ __forceinline__ void append(bool sel, uint64_t key, int64_t i, unsigned long long *__restrict__ cnt,
                                       unsigned long long limit, uint64_t *__restrict__ keys,
                                       uint64_t *__restrict__ vals)
{
    const unsigned bm = __ballot_sync(0xffffffffu, sel);
    if (!bm) return;
    const int lane = threadIdx.x & 31, leader = __ffs(bm) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(cnt, (unsigned long long)__popc(bm));
    base = __shfl_sync(0xffffffffu, base, leader);
    const unsigned long long at = base + __popc(bm & ((1u << lane) - 1u));
    if (sel && at < limit) {               // the host checks the count against the histogram's
        keys[at] = key;
        vals[at] = (uint64_t)i;
    }
}

__global__ void gather_buckets(const uint8_t *__restrict__ text, int64_t n, int blo, int bhi,
                               unsigned long long *__restrict__ cnt, unsigned long long limit,
                               uint64_t *__restrict__ keys, uint64_t *__restrict__ vals)
{
    const int64_t m = n + 1;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t w = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); w * 32 < m; w += warps) {
        const int64_t i = w * 32 + (threadIdx.x & 31);
        bool sel = false;
        if (i < m) {
            const int b = bucket_of(text, n, i);
            sel = b >= blo && b < bhi;
        }
        append(sel, sel ? key21(text, n, i) : 0, i, cnt, limit, keys, vals);
    }
}

__global__ void gather_ranks(const uint64_t *__restrict__ rank, int64_t m, int64_t h, uint64_t rlo, uint64_t rhi,
                             int rbits, unsigned long long *__restrict__ cnt, unsigned long long limit,
                             uint64_t *__restrict__ keys, uint64_t *__restrict__ vals)
{
    const uint64_t mask = (1ull << rbits) - 1;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t w = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); w * 32 < m; w += warps) {
        const int64_t i = w * 32 + (threadIdx.x & 31);
        bool sel = false;
        uint64_t key = 0;
        if (i < m) {
            const uint64_t r = rank[i];
            sel = !(r & kAlone) && r >= rlo && r < rhi;
            if (sel) key = (r - rlo) << rbits | (i + h < m ? rank[i + h] & mask : 0);
        }
        append(sel, key, i, cnt, limit, keys, vals);
    }
}

// Row j of the sorted chunk ends a group when the key above bit `from` differs from row j+1's;
// out[N-1-j] = N-1-j there, else 0, so an inclusive max-scan of out gives each row, read back at
// N-1-j, N-1 minus the last row of its group.
__global__ void tails_rev(const uint64_t *__restrict__ key, int64_t N, int from, uint32_t *__restrict__ out)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < N; j += (int64_t)gridDim.x * blockDim.x) {
        const bool tail = j + 1 == N || (key[j] >> from) != (key[j + 1] >> from);
        out[N - 1 - j] = tail ? (uint32_t)(N - 1 - j) : 0u;
    }
}

// New ranks of a sorted chunk, the position of the last row of each suffix's group: base + that
// row in round 0 (base = the chunk's first position); later, the old group's rank (its last row)
// less the rows of the old group after the new group's last row.
__global__ void write_ranks(const uint64_t *__restrict__ key, const uint64_t *__restrict__ val, int64_t N,
                            const uint32_t *__restrict__ ek, const uint32_t *__restrict__ eo, int rbits,
                            uint64_t base, int round0, uint64_t *__restrict__ rank,
                            unsigned long long *__restrict__ n_open)
{
    unsigned open = 0;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < N; j += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = key[j];
        const int64_t end = N - 1 - (int64_t)ek[N - 1 - j];
        const bool alone = end == j && (j == 0 || key[j - 1] != k);
        uint64_t r;
        if (round0) {
            r = base + (uint64_t)end;
        } else {
            const int64_t oend = N - 1 - (int64_t)eo[N - 1 - j];
            r = base + (k >> rbits) - (uint64_t)(oend - end);
        }
        rank[val[j]] = r | (alone ? kAlone : 0);
        open += !alone;
    }
    open = __reduce_add_sync(0xffffffffu, open);
    if ((threadIdx.x & 31) == 0 && open) atomicAdd(n_open, (unsigned long long)open);
}

// BWT symbols (2 bits, 16 to a word, first symbol in the top bits) and sampled rows, from the ranks
__global__ void bwt_from_ranks(const uint8_t *__restrict__ text, const uint64_t *__restrict__ rank, int64_t n,
                               uint64_t primary, int sa_intv, uint32_t *__restrict__ bwt, uint64_t *__restrict__ sa)
{
    const int64_t m = n + 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t r = rank[i] & ~kAlone;
        if (r % (uint64_t)sa_intv == 0) sa[r / (uint64_t)sa_intv] = (uint64_t)i;
        if (i == 0) continue;
        const uint64_t pos = r - (r > primary);
        atomicOr(&bwt[pos >> 4], (uint32_t)text[i - 1] << ((15 - (pos & 15)) << 1));
    }
}

}  // namespace

extern "C" int bsb_build_bwt(bsb_ctx *ctx, const uint8_t *pac, int64_t l_pac, int sa_intv, int64_t chunk,
                             uint32_t *bwt, uint64_t *primary, uint64_t *sa)
{
    if (!ctx) return BSB_EINVAL;
    if (!pac || !bwt || !primary || !sa || l_pac < 1 || sa_intv < 1)
        return bsb_fail(ctx, BSB_EINVAL, "NULL argument, empty pac or SA interval < 1");
    const int64_t n = 2 * l_pac, m = n + 1;
    int rbits = 1;
    while (rbits < 62 && (1ll << rbits) < m) ++rbits;           // ranks 0 .. m-1 < 2^rbits
    if (rbits > 40) return bsb_fail(ctx, BSB_ETOOLONG, "text of %lld symbols", (long long)n);
    const uint64_t max_range = rbits >= 63 ? 1 : 1ull << (63 - rbits);   // rank span of one chunk (bit 63 spare)
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    cudaStream_t st = ctx->stream;
    const size_t pb = (size_t)(l_pac + 3) / 4;
    const int64_t n_words = (n + 15) / 16, n_sa = (n + sa_intv) / sa_intv;
    DevBuf d_pac, d_text, d_rank, d_hist, d_cnt, k0, k1, v0, v1, s0, s1, d_tmp;
    if ((rc = bsb_cuda(ctx, cudaMalloc(&d_text.p, (size_t)n + 64), "BWT build: text")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&d_rank.p, 8 * (size_t)m), "BWT build: ranks")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&d_hist.p, 8 * (size_t)std::max(kBuckets, 1 << kBinBits)),
                       "BWT build: histogram")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&d_cnt.p, 64), "BWT build: counters")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&d_pac.p, pb + 16), "BWT build: pac")))
        return rc;
    const int grid = ctx->n_sm * 8;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(d_pac.p, pac, pb, cudaMemcpyHostToDevice, st), "BWT build: H2D pac")))
        return rc;
    text_kernel<<<grid, 256, 0, st>>>((const uint8_t *)d_pac.p, l_pac, (uint8_t *)d_text.p);
    if ((rc = bsb_cuda(ctx, cudaStreamSynchronize(st), "BWT build: text"))) return rc;
    cudaFree(d_pac.p);
    d_pac.p = nullptr;
    // the chunk: as many suffixes as the free memory holds at 44 bytes each (keys, suffixes, group rows
    // and sort scratch) less 3 GB, at most 2^31 - 1
    size_t fr = 0, tot = 0;
    if ((rc = bsb_cuda(ctx, cudaMemGetInfo(&fr, &tot), "BWT build: memory"))) return rc;
    int64_t cap = (int64_t)((fr > ((size_t)3 << 30) ? fr - ((size_t)3 << 30) : 0) / 44);
    cap = std::min<int64_t>(cap, 0x7fffffffLL);
    cap = std::min<int64_t>(cap, m);
    if (chunk > 0) cap = std::min<int64_t>(cap, chunk);
    if (cap < std::min<int64_t>(m, 32)) return bsb_fail(ctx, BSB_ENOMEM, "BWT build: no room for a sort chunk");
    size_t tmp_sort = 0, tmp_scan = 0;
    {
        cub::DoubleBuffer<uint64_t> kk((uint64_t *)nullptr, (uint64_t *)nullptr);
        cub::DoubleBuffer<uint64_t> vv((uint64_t *)nullptr, (uint64_t *)nullptr);
        if (cub::DeviceRadixSort::SortPairs(nullptr, tmp_sort, kk, vv, (int)cap, 0, 64, st) != cudaSuccess ||
            cub::DeviceScan::InclusiveScan(nullptr, tmp_scan, (uint32_t *)nullptr, (uint32_t *)nullptr,
                                           cuda::maximum<>(), (int)cap, st) != cudaSuccess)
            return bsb_fail(ctx, BSB_ECUDA, "BWT build: sort set-up");
    }
    const size_t tmp_bytes = std::max(tmp_sort, tmp_scan);
    if ((rc = bsb_cuda(ctx, cudaMalloc(&k0.p, 8 * (size_t)cap), "BWT build: keys")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&k1.p, 8 * (size_t)cap), "BWT build: keys")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&v0.p, 8 * (size_t)cap), "BWT build: suffixes")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&v1.p, 8 * (size_t)cap), "BWT build: suffixes")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&s0.p, 4 * (size_t)cap), "BWT build: group rows")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&s1.p, 4 * (size_t)cap), "BWT build: group rows")) ||
        (rc = bsb_cuda(ctx, cudaMalloc(&d_tmp.p, tmp_bytes + 256), "BWT build: sort scratch")))
        return rc;
    const uint8_t *text = (const uint8_t *)d_text.p;
    uint64_t *rank = (uint64_t *)d_rank.p;
    unsigned long long *cnt = (unsigned long long *)d_cnt.p, *hist = (unsigned long long *)d_hist.p;

    // sorts the gathered chunk of N suffixes on key bits [0, end_bit) and writes their ranks
    unsigned long long h_cnt[2];
    auto sort_chunk = [&](int64_t N, int end_bit, int round0, uint64_t base) -> int {
        cub::DoubleBuffer<uint64_t> keys((uint64_t *)k0.p, (uint64_t *)k1.p);
        cub::DoubleBuffer<uint64_t> vals((uint64_t *)v0.p, (uint64_t *)v1.p);
        size_t t = 0;
        int r;
        if ((r = bsb_cuda(ctx, cub::DeviceRadixSort::SortPairs(nullptr, t, keys, vals, (int)N, 0, end_bit, st),
                          "BWT build: sort set-up")))
            return r;
        if (t > tmp_bytes) return bsb_fail(ctx, BSB_ENOMEM, "BWT build: sort scratch of %zu bytes", t);
        t = tmp_bytes;
        if ((r = bsb_cuda(ctx, cub::DeviceRadixSort::SortPairs(d_tmp.p, t, keys, vals, (int)N, 0, end_bit, st),
                          "BWT build: sort")))
            return r;
        const int g = (int)std::min<int64_t>((N + 255) / 256, (int64_t)ctx->n_sm * 16);
        uint32_t *ek = (uint32_t *)s0.p, *eo = (uint32_t *)s1.p;
        tails_rev<<<g, 256, 0, st>>>(keys.Current(), N, 0, ek);
        t = tmp_bytes;
        if ((r = bsb_cuda(ctx, cub::DeviceScan::InclusiveScan(d_tmp.p, t, ek, ek, cuda::maximum<>(), (int)N, st),
                          "BWT build: group scan")))
            return r;
        if (!round0) {
            tails_rev<<<g, 256, 0, st>>>(keys.Current(), N, rbits, eo);
            t = tmp_bytes;
            if ((r = bsb_cuda(ctx, cub::DeviceScan::InclusiveScan(d_tmp.p, t, eo, eo, cuda::maximum<>(), (int)N,
                                                                  st), "BWT build: group scan")))
                return r;
        }
        write_ranks<<<g, 256, 0, st>>>(keys.Current(), vals.Current(), N, ek, eo, rbits, base, round0, rank,
                                       cnt + 1);
        return bsb_cuda(ctx, cudaGetLastError(), "BWT build: ranks");
    };

    // the gather of a chunk appended exactly the suffixes its histogram counted
    auto gathered = [&](uint64_t N) -> int {
        unsigned long long got = 0;
        int r;
        if ((r = bsb_cuda(ctx, cudaMemcpyAsync(&got, cnt, 8, cudaMemcpyDeviceToHost, st), "BWT build: count")) ||
            (r = bsb_cuda(ctx, cudaStreamSynchronize(st), "BWT build: gather")))
            return r;
        return got == N ? 0 : bsb_fail(ctx, BSB_EINVAL, "BWT build: gathered %llu suffixes, counted %llu", got,
                                       (unsigned long long)N);
    };

    // round 0: buckets of the first five symbols, chunks of whole buckets, 21-symbol keys
    std::vector<unsigned long long> bh(kBuckets);
    if ((rc = bsb_cuda(ctx, cudaMemsetAsync(hist, 0, 8 * (size_t)kBuckets, st), "BWT build: histogram")) ||
        (rc = bsb_cuda(ctx, cudaMemsetAsync(cnt, 0, 16, st), "BWT build: counters")))
        return rc;
    bucket_hist<<<grid, 256, 0, st>>>(text, n, hist);
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(bh.data(), hist, 8 * (size_t)kBuckets, cudaMemcpyDeviceToHost, st),
                       "BWT build: histogram")) ||
        (rc = bsb_cuda(ctx, cudaStreamSynchronize(st), "BWT build: histogram")))
        return rc;
    {
        uint64_t pos = 0;
        for (int b = 0; b < kBuckets;) {
            if ((int64_t)bh[b] > cap) return bsb_fail(ctx, BSB_ENOMEM, "BWT build: bucket of %llu suffixes", bh[b]);
            int e = b;
            uint64_t N = 0;
            while (e < kBuckets && N + bh[e] <= (uint64_t)cap) N += bh[e++];
            if (N) {
                if ((rc = bsb_cuda(ctx, cudaMemsetAsync(cnt, 0, 8, st), "BWT build: counters"))) return rc;
                gather_buckets<<<grid, 256, 0, st>>>(text, n, b, e, cnt, (unsigned long long)cap, (uint64_t *)k0.p,
                                                     (uint64_t *)v0.p);
                if ((rc = gathered(N)) || (rc = sort_chunk((int64_t)N, 63, 1, pos))) return rc;
            }
            pos += N;
            b = e;
        }
    }
    // rounds 1, 2, ...: the suffixes whose group has more members, by rank bins
    const int shift = rbits > kBinBits ? rbits - kBinBits : 0;
    const int n_bins = (int)(((uint64_t)(m - 1) >> shift) + 1);
    std::vector<unsigned long long> rh(n_bins);
    for (int64_t h = kPrefixSyms, round = 1;; h *= 2, ++round) {
        if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(h_cnt, cnt, 16, cudaMemcpyDeviceToHost, st), "BWT build: count")) ||
            (rc = bsb_cuda(ctx, cudaStreamSynchronize(st), "BWT build: round")))
            return rc;
        if (h_cnt[1] == 0) break;                                   // every suffix is alone: sorted
        if (round > 40) return bsb_fail(ctx, BSB_EINVAL, "BWT build: no convergence");
        if ((rc = bsb_cuda(ctx, cudaMemsetAsync(hist, 0, 8 * (size_t)n_bins, st), "BWT build: histogram")) ||
            (rc = bsb_cuda(ctx, cudaMemsetAsync(cnt, 0, 16, st), "BWT build: counters")))
            return rc;
        rank_hist<<<grid, 256, 0, st>>>(rank, m, shift, n_bins, hist);
        if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(rh.data(), hist, 8 * (size_t)n_bins, cudaMemcpyDeviceToHost, st),
                           "BWT build: histogram")) ||
            (rc = bsb_cuda(ctx, cudaStreamSynchronize(st), "BWT build: histogram")))
            return rc;
        const uint64_t bins_per_range = std::max<uint64_t>(1, max_range >> shift);
        for (int b = 0; b < n_bins;) {
            if ((int64_t)rh[b] > cap) return bsb_fail(ctx, BSB_ENOMEM, "BWT build: rank bin of %llu suffixes", rh[b]);
            int e = b;
            uint64_t N = 0;
            while (e < n_bins && N + rh[e] <= (uint64_t)cap && (uint64_t)(e - b) < bins_per_range) N += rh[e++];
            if (N) {
                const uint64_t rlo = (uint64_t)b << shift, rhi = (uint64_t)e << shift;
                int span = 1;
                while (span < 63 - rbits && (1ull << span) < rhi - rlo) ++span;
                if ((rc = bsb_cuda(ctx, cudaMemsetAsync(cnt, 0, 8, st), "BWT build: counters"))) return rc;
                gather_ranks<<<grid, 256, 0, st>>>(rank, m, h, rlo, rhi, rbits, cnt, (unsigned long long)cap,
                                                   (uint64_t *)k0.p, (uint64_t *)v0.p);
                if ((rc = gathered(N)) || (rc = sort_chunk((int64_t)N, std::min(64, rbits + span), 0, rlo)))
                    return rc;
            }
            b = e;
        }
    }
    // the BWT without the row of suffix 0, and the sampled rows
    uint64_t r0 = 0;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(&r0, rank, 8, cudaMemcpyDeviceToHost, st), "BWT build: primary")) ||
        (rc = bsb_cuda(ctx, cudaStreamSynchronize(st), "BWT build: primary")))
        return rc;
    *primary = r0 & ~kAlone;
    uint32_t *d_bwt = (uint32_t *)k0.p;
    uint64_t *d_sa = (uint64_t *)k1.p;
    DevBuf big_bwt, big_sa;                   // when a sort buffer is too small for them
    if ((int64_t)(8 * cap) < 4 * n_words) {
        if ((rc = bsb_cuda(ctx, cudaMalloc(&big_bwt.p, 4 * (size_t)n_words), "BWT build: BWT"))) return rc;
        d_bwt = (uint32_t *)big_bwt.p;
    }
    if (cap < n_sa) {
        if ((rc = bsb_cuda(ctx, cudaMalloc(&big_sa.p, 8 * (size_t)n_sa), "BWT build: sampled SA"))) return rc;
        d_sa = (uint64_t *)big_sa.p;
    }
    if ((rc = bsb_cuda(ctx, cudaMemsetAsync(d_bwt, 0, 4 * (size_t)n_words, st), "BWT build: BWT"))) return rc;
    bwt_from_ranks<<<grid, 256, 0, st>>>(text, rank, n, *primary, sa_intv, d_bwt, d_sa);
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(bwt, d_bwt, 4 * (size_t)n_words, cudaMemcpyDeviceToHost, st),
                       "BWT build: D2H BWT")) ||
        (rc = bsb_cuda(ctx, cudaMemcpyAsync(sa, d_sa, 8 * (size_t)n_sa, cudaMemcpyDeviceToHost, st),
                       "BWT build: D2H sampled SA")))
        return rc;
    return bsb_cuda(ctx, cudaStreamSynchronize(st), "BWT build");
}
