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

#include "ksw_group.cuh"

namespace {

// Tiles: G lanes per job (32/G jobs per warp) x C query columns per lane;
// a tile holds queries of up to G*C - 1 bases (columns 0..qlen).
struct Tile { int G, C; };
constexpr Tile kTiles[] = {
    {4, 1}, {4, 2}, {4, 3}, {4, 4}, {4, 5}, {4, 6}, {4, 7}, {4, 8},      // qlen <= 31
    {8, 5}, {8, 6}, {8, 7}, {8, 8},                                      // <= 63
    {16, 5}, {16, 6}, {16, 7}, {16, 8},                                  // <= 127
    {32, 5}, {32, 6}, {32, 7}, {32, 8},                                  // <= 255
    {32, 10}, {32, 12}, {32, 16}, {32, 24}, {32, 32}};                   // <= 1023
constexpr int kNumBins = sizeof(kTiles) / sizeof(kTiles[0]);
constexpr int kClasses = 128;           // cost classes within a bin
constexpr int kBlock = 128;             // threads per block (4 warps)

// Bin of the smallest tile that holds columns 0..qlen.
__host__ __device__ inline int tile_bin(int qlen)
{
    const int need = qlen + 1;
    if (need <= 32) return (need + 3) / 4 - 1;
    if (need <= 64) return 8 + (need + 7) / 8 - 5;
    if (need <= 128) return 12 + (need + 15) / 16 - 5;
    if (need <= 256) return 16 + (need + 31) / 32 - 5;
    if (need <= 320) return 20;
    if (need <= 384) return 21;
    if (need <= 512) return 22;
    if (need <= 768) return 23;
    if (need <= 1024) return 24;
    return -1;
}

// Persistent per-bin kernel.  Each group of G lanes pulls job indices from
// counter[bin] and runs its jobs row by row; the warp leaves when the queue is
// empty and every group is done.
template <int C, int G>
__global__ void __launch_bounds__(kBlock)
ksw_group_kernel(KswParams P, const bsb_ext_job_t *__restrict__ jobs, const uint8_t *__restrict__ seq,
                 const int32_t *__restrict__ order, const int32_t *__restrict__ bin_start, int bin,
                 int *__restrict__ counter, bsb_ext_out_t *__restrict__ out, int64_t *__restrict__ cells)
{
    ksw_group_run<C, G>(P, jobs, seq, order, bin_start[bin], bin_start[bin + 1], counter + bin, out, cells);
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

template <int C, int G>
cudaError_t launch_bin(const KswParams &P, const bsb_ext_job_t *jobs, const uint8_t *seq,
                       const int32_t *order, const int32_t *bin_start, int bin, int *counter,
                       bsb_ext_out_t *out, int64_t *cells, int n_sm, cudaStream_t st)
{
    static int blocks_per_sm = 0;
    if (!blocks_per_sm) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, ksw_group_kernel<C, G>, kBlock, 0);
        if (e != cudaSuccess) return e;
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    ksw_group_kernel<C, G><<<n_sm * blocks_per_sm, kBlock, 0, st>>>(P, jobs, seq, order, bin_start, bin, counter, out,
                                                                      cells);
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
        cudaError_t e = launch_bin<kTiles[I].C, kTiles[I].G>(P, jobs, seq, order, bin_start, I, counter, out, cells,
                                                             n_sm, st);
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

int ksw_max_qlen() { return kTiles[kNumBins - 1].G * kTiles[kNumBins - 1].C - 1; }

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
