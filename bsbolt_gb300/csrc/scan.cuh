// scan.cuh -- exclusive prefix sum of int32 counts into int64 offsets, off[n] = total.
//
// Three launches: per-tile sums (coalesced, one block per tile of kScanTile counts),
// one block scanning the tile sums into tile offsets, then each tile scanned in its
// block and shifted by its offset.  tmp holds scan_tmp_words(n) int64.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace scan_detail {
namespace {     // each translation unit that includes this gets its own kernels

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

// Block-wide inclusive scan of one value per thread (256 threads).
__device__ __forceinline__ int64_t block_inclusive(int64_t v, int64_t *warp_tot)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int64_t u = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += u;
    }
    if (lane == 31) warp_tot[wid] = v;
    __syncthreads();
    if (wid == 0) {
        int64_t w = lane < kScanThreads / 32 ? warp_tot[lane] : 0;
#pragma unroll
        for (int d = 1; d < kScanThreads / 32; d <<= 1) {
            const int64_t u = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= d) w += u;
        }
        if (lane < kScanThreads / 32) warp_tot[lane] = w;
    }
    __syncthreads();
    const int64_t before = wid ? warp_tot[wid - 1] : 0;
    __syncthreads();
    return v + before;
}

__global__ void __launch_bounds__(kScanThreads) tile_sums(const int *__restrict__ cnt, int64_t n,
                                                           int64_t *__restrict__ sums)
{
    __shared__ int64_t wt[kScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    int64_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + k * kScanThreads + threadIdx.x;
        if (i < n) s += cnt[i];
    }
    const int64_t incl = block_inclusive(s, wt);
    if (threadIdx.x == kScanThreads - 1) sums[blockIdx.x] = incl;
}

// One block: exclusive scan of the tile sums in place; the total goes to *total.
__global__ void __launch_bounds__(kScanThreads) tile_offsets(int64_t *__restrict__ sums, int64_t n_tiles,
                                                              int64_t *__restrict__ total)
{
    __shared__ int64_t wt[kScanThreads / 32];
    int64_t carry = 0;
    for (int64_t b = 0; b < n_tiles; b += kScanThreads) {
        const int64_t i = b + threadIdx.x;
        const int64_t v = i < n_tiles ? sums[i] : 0;
        const int64_t incl = block_inclusive(v, wt);
        if (i < n_tiles) sums[i] = carry + incl - v;
        carry += wt[kScanThreads / 32 - 1];        // the block's total
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kScanThreads) tile_scan(const int *__restrict__ cnt, int64_t n,
                                                           const int64_t *__restrict__ tile_off,
                                                           int64_t *__restrict__ off)
{
    __shared__ int64_t wt[kScanThreads / 32];
    // thread t owns kScanItems consecutive counts of the tile (loaded through shared memory
    // in coalesced order)
    __shared__ int sh[kScanTile];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + k * kScanThreads + threadIdx.x;
        sh[k * kScanThreads + threadIdx.x] = i < n ? cnt[i] : 0;
    }
    __syncthreads();
    int v[kScanItems];
    int64_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = sh[threadIdx.x * kScanItems + k];
        s += v[k];
    }
    const int64_t excl = block_inclusive(s, wt) - s + tile_off[blockIdx.x];
    int64_t acc = excl;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + threadIdx.x * kScanItems + k;
        if (i < n) off[i] = acc;
        acc += v[k];
    }
}

}  // namespace
}  // namespace scan_detail

inline int64_t scan_tmp_words(int64_t n)
{
    return (n + scan_detail::kScanTile - 1) / scan_detail::kScanTile + 1;
}

// off[0..n) = exclusive prefix sums of cnt, off[n] = the total.
inline cudaError_t scan_i32_i64(const int *cnt, int64_t n, int64_t *off, int64_t *tmp, cudaStream_t st)
{
    using namespace scan_detail;
    const int64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles > 0) tile_sums<<<(unsigned)tiles, kScanThreads, 0, st>>>(cnt, n, tmp);
    tile_offsets<<<1, kScanThreads, 0, st>>>(tmp, tiles, off + n);
    if (tiles > 0) tile_scan<<<(unsigned)tiles, kScanThreads, 0, st>>>(cnt, n, tmp, off);
    return cudaGetLastError();
}
