// sa_build.cu -- the suffix array of BWA's index text, built on the GPU.
//
// bwa index sorts the suffixes of the forward 2-bit pac followed by its reverse complement
// (2*l_pac symbols, bntseq.c / bwtindex.c) with a sentinel '$' that sorts before every base;
// the BWT, the occurrence array and the sampled SA (.bwt, .sa) are read off that order.
// On the host (host_index.c) an SA-IS with 32-bit indexes does this up to 2^31 symbols and
// takes minutes per billion; here prefix doubling runs on device radix sorts (CUB, part of
// the CUDA toolkit): every suffix is first keyed by its next 21 symbols (3 bits each, 0 past
// the end), sorted, and given the rank of its group's first row; then each round keys suffix
// i by (rank[i], rank[i + h]) and sorts again, h = 21, 42, 84, ... until every rank is
// distinct.  Suffixes whose first h symbols reach the sentinel are already alone in their
// group, so rank[i + h] past the end can be anything.  Ranks are 32-bit: up to 2^32 - 1
// suffixes (texts below 2^32 - 1 symbols, references up to ~1.07 Gb converted both ways).
// Device memory: ~33 bytes per symbol at the peak (two 8-byte key and two 4-byte index
// buffers of the sort, the rank array, the text), all freed before returning.

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
