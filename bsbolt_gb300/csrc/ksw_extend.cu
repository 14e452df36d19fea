// ksw_extend.cu -- batched ksw_extend2 for sm_103a: the scheduler.
//
// Bit-exact restatement of the reference banded extension
// (bsbolt/External/BWA/ksw.c:380-479).  The DP itself is ksw_group.cuh: a
// group of G lanes runs one job row by row, 32/G jobs per warp.
//
// Why row-parallel and not an anti-diagonal wavefront: the reference decides
// each row's band [beg,end) from the complete previous row (the shrink to
// non-zero cells, ksw.c:466-469), stops on a zero row (ksw.c:454) and tests
// z-drop per target row (ksw.c:458-464).  A wavefront would have to run rows
// whose band is not known yet.  Instead a group computes a whole row at once:
//   * lane L of the group owns query columns [L*C, L*C+C) in registers;
//   * M and E depend only on the previous row and are computed per cell;
//   * F(i,j+1) = max(F(i,j) - e_ins, max(M(i,j) - oe_ins, 0)) is a max-plus
//     recurrence along the row: each lane runs it over its own columns, and
//     a group scan of the lane maps x -> max(x - e_ins*C, F_lane) supplies
//     every lane's carry-in (one __shfl_up_sync ladder per row);
//   * the row maximum, its last column, and the first/last non-zero cell of
//     the shrink are group reductions.
// The register file holds the reference's whole eh[] array, including cells
// outside the current band: the band may grow back over them and read stale
// values, exactly as the reference does.
//
// Scheduling (the plain schedule): each job gets the tile shape the tile map
// assigns to its query length (ksw_tiles.cuh), and within a shape jobs are
// issued longest-bound-first (qlen x min(tlen, qlen+w), or a caller supplied
// cost key); each shape runs as a persistent kernel whose groups pull jobs
// from a device counter.  Shapes with an even C run their jobs on 16-bit cells,
// two per register (ksw_group16.cuh); a job whose scores could leave 16 bits
// (h0 + qlen * max(mat) > kPack16MaxH) is binned last in its shape and runs on
// the 32-bit kernel.  Results never depend on the shape, the cell width or the
// order.

#include <climits>
#include <cstdio>

#include "ksw_group16.cuh"
#include "ksw_tiles.cuh"

__constant__ KswTileMap c_default_tile_map = kDefaultTileMap;

namespace {

constexpr int kClasses = 128;           // cost classes within a tile shape; the last one holds the
                                        // jobs that need 32-bit cells
constexpr int kWideClass = kClasses - 1;

__device__ __forceinline__ int cost_class(uint32_t key)
{
    // 4 classes per power of two; class 0 = cheapest
    if (key == 0) return 0;
    const int msb = 31 - __clz(key);
    const int frac = msb >= 2 ? (int)((key >> (msb - 2)) & 3) : (int)((key << (2 - msb)) & 3);
    const int c = msb * 4 + frac;
    return c < kWideClass ? c : kWideClass - 1;
}

// Shapes with a 16-bit kernel (tile_has_pack16), as a bit set.
constexpr uint64_t pack16_tiles()
{
    uint64_t m = 0;
    for (int t = 0; t < kNumTiles; ++t)
        if (tile_has_pack16(kTileList[t].C)) m |= 1ull << t;
    return m;
}
constexpr uint64_t kPack16Tiles = pack16_tiles();

// Histogram of (tile, class) keys.  Tiles are major; within a tile, classes
// are laid out most expensive first so an ascending scan issues longest-first.
// A job that fails the preconditions (the host entry checks them; the device
// entry cannot) gets the reject key kRejectKey: it is counted, never issued,
// and its output is left untouched.
constexpr int kRejectKey = kNumTiles * kClasses;
constexpr int kHistSlots = kNumTiles * kClasses + 1;
constexpr int kScanThreads = 1024;

__global__ void ksw_sched_hist(const bsb_ext_job_t *__restrict__ jobs, int n, long long seq_bytes,
                               const int32_t *__restrict__ cost, const uint8_t *__restrict__ map, int pack16,
                               int mat_max, int *__restrict__ hist, int32_t *__restrict__ key_out)
{
    __shared__ int sh[kHistSlots];
    for (int i = threadIdx.x; i < kHistSlots; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const bsb_ext_job_t jb = jobs[i];
        const bool ok = jb.qlen >= 0 && jb.qlen < kMaxNeed && jb.tlen >= 0 && jb.w >= 0 && jb.h0 > 0 &&
                        jb.h0 <= (1 << 20) && jb.flags == 0 && jb.qoff >= 0 && jb.toff >= 0 &&
                        jb.qoff + jb.qlen <= seq_bytes && jb.toff + jb.tlen <= seq_bytes;
        int key;
        if (!ok) {
            key = kRejectKey;
        } else {
            const int need = jb.qlen + 1;
            const int t = map ? map[need] : c_default_tile_map.tile[need];
            uint32_t k;
            if (cost) k = (uint32_t)max(cost[i], 0);
            else {
                const long long span = min((long long)jb.tlen, (long long)jb.qlen + jb.w);
                const long long c = (long long)jb.qlen * max(span, 0LL);
                k = (uint32_t)min(c, (long long)0x7fffffff);
            }
            const bool wide = pack16 && (kPack16Tiles >> t & 1) &&
                              (long long)jb.h0 + (long long)jb.qlen * mat_max > kPack16MaxH;
            key = t >= kNumTiles ? kRejectKey
                  : wide         ? t * kClasses + kWideClass
                                 : t * kClasses + (kWideClass - 1 - cost_class(k));
        }
        key_out[i] = key;
        atomicAdd(&sh[key], 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kHistSlots; i += blockDim.x)
        if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// Exclusive scan of the histogram (one block: a contiguous chunk per thread,
// then a scan of the chunk totals) -> cursors and, per tile t, the ranges of its
// launches: ranges[6t ..] = {start, wide start | wide start, end | start, end}
// (the 16-bit kernel, the 32-bit kernel for the wide class, or one 32-bit kernel
// for the whole tile).  rejected[0] counts the rejected jobs.
constexpr int kRangeInts = 6;
__global__ void __launch_bounds__(kScanThreads)
ksw_sched_scan(const int *__restrict__ hist, int *__restrict__ cursor, int32_t *__restrict__ ranges,
               int *__restrict__ rejected)
{
    constexpr int kChunk = (kHistSlots + kScanThreads - 1) / kScanThreads;
    __shared__ int tot[kScanThreads];
    const int t = threadIdx.x, lo = t * kChunk;
    int v[kChunk];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kChunk; ++k) {
        v[k] = lo + k < kHistSlots ? hist[lo + k] : 0;
        s += v[k];
    }
    tot[t] = s;
    __syncthreads();
    for (int d = 1; d < kScanThreads; d <<= 1) {      // inclusive Hillis-Steele scan of the totals
        const int add = t >= d ? tot[t - d] : 0;
        __syncthreads();
        tot[t] += add;
        __syncthreads();
    }
    int acc = t ? tot[t - 1] : 0;
#pragma unroll
    for (int k = 0; k < kChunk; ++k) {
        const int i = lo + k;
        if (i < kHistSlots) {
            cursor[i] = acc;
            const int tile = i / kClasses, cls = i % kClasses;
            if (cls == 0) {
                if (tile < kNumTiles) ranges[kRangeInts * tile] = ranges[kRangeInts * tile + 4] = acc;
                if (tile > 0) ranges[kRangeInts * (tile - 1) + 3] = ranges[kRangeInts * (tile - 1) + 5] = acc;
            }
            if (cls == kWideClass && tile < kNumTiles)
                ranges[kRangeInts * tile + 1] = ranges[kRangeInts * tile + 2] = acc;
            if (i == kRejectKey) rejected[0] = tot[kScanThreads - 1] - acc;
        }
        acc += v[k];
    }
}

__global__ void ksw_sched_scatter(const int32_t *__restrict__ key, int n, int *__restrict__ cursor,
                                  int32_t *__restrict__ order)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int pos = atomicAdd(&cursor[key[i]], 1);
        order[pos] = i;
    }
}

}  // namespace

static_assert(kRejectKey % kClasses == 0, "the reject slot starts a bin");

// scratch layout (int32 words): counter[3*kNumTiles] | rejected[1] | hist[kHistSlots] |
//   cursor[kHistSlots] | ranges[kRangeInts*kNumTiles] | (256-byte aligned) key[n] | order[n]
static size_t fixed_bytes()
{
    size_t fixed = sizeof(int) * (3 * kNumTiles + 1 + 2 * kHistSlots + kRangeInts * kNumTiles);
    return (fixed + 255) & ~(size_t)255;
}

size_t ksw_scratch_bytes(int64_t n) { return fixed_bytes() + sizeof(int32_t) * 2 * (size_t)n + 256; }

int ksw_max_qlen() { return kMaxNeed - 1; }

int64_t ksw_concurrent_below() { return (int64_t)1 << 20; }

int *ksw_rejected_counter(void *scratch) { return (int *)scratch + 3 * kNumTiles; }

const uint8_t *ksw_default_tile_map() { return kDefaultTileMap.tile; }

int ksw_tile_shape(int t, int *G, int *C)
{
    if (t < 0 || t >= kNumTiles) return -1;
    *G = kTileList[t].G;
    *C = kTileList[t].C;
    return 0;
}

uint64_t ksw_map_tiles(const uint8_t *map)
{
    uint64_t m = 0;
    for (int need = 1; need <= kMaxNeed; ++need) m |= 1ull << map[need];
    return m;
}

cudaError_t ksw_launch(const KswParams &P, const bsb_ext_job_t *d_jobs, int64_t n, int64_t seq_bytes,
                       const uint8_t *d_seq, const int32_t *d_cost, const uint8_t *d_map, uint64_t tiles,
                       bsb_ext_out_t *d_out, int64_t *d_cells, void *scratch, int n_sm, cudaStream_t st,
                       cudaEvent_t ev0, cudaEvent_t ev1, const cudaEvent_t *tile_ev, const KswStreams *ms)
{
    char *p = (char *)scratch;
    int *counter = (int *)p;                // 3 per tile: 16-bit range, wide range, whole tile
    int *rejected = counter + 3 * kNumTiles;
    int *hist = rejected + 1;
    int *cursor = hist + kHistSlots;
    int32_t *ranges = cursor + kHistSlots;
    int32_t *key = (int32_t *)(p + fixed_bytes());
    int32_t *order = key + n;
    // 16-bit cells need every value of the packed arithmetic inside 16 bits: penalties
    // and their multiples by a lane's column count stay small, and scores at most
    // kPack16MaxScore (h0 + qlen * max score is checked per job)
    KswParams Q = P;
    Q.pack16 = P.o_del + P.e_del <= 8000 && P.o_ins + P.e_ins <= 8000 && P.e_del <= 500 && P.e_ins <= 500 &&
               P.mat_max <= kPack16MaxScore;
    cudaError_t e;
    if (ev0) cudaEventRecord(ev0, st);
    e = cudaMemsetAsync(scratch, 0, sizeof(int) * (3 * kNumTiles + 1 + kHistSlots), st);
    if (e != cudaSuccess) return e;
    if (n > 0) {
        const int nb = (int)min((int64_t)n_sm * 8, (n + 255) / 256);
        ksw_sched_hist<<<nb, 256, 0, st>>>(d_jobs, (int)n, (long long)seq_bytes, d_cost, d_map, Q.pack16,
                                           Q.mat_max, hist, key);
        ksw_sched_scan<<<1, kScanThreads, 0, st>>>(hist, cursor, ranges, rejected);
        ksw_sched_scatter<<<nb, 256, 0, st>>>(key, (int)n, cursor, order);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        // Small batches: the shapes run on four streams, so the next shape's blocks fill
        // the SMs a finishing shape leaves during its tail.  Large batches keep one stream
        // (the tails are a small part of them, and each shape is timed alone).
        const bool conc = ms && n < ksw_concurrent_below();
        if (conc) {
            cudaEventRecord(ms->fork, st);
            for (int a = 0; a < BSB_AUX_STREAMS; ++a) cudaStreamWaitEvent(ms->aux[a], ms->fork, 0);
        }
        int k = 0;
        for (int t = 0; t < kNumTiles; ++t) {
            if (!(tiles >> t & 1)) continue;
            KswTileLaunch f = ksw_tile_launcher(t), f16 = Q.pack16 ? ksw_tile16_launcher(t) : nullptr;
            if (!f) return cudaErrorInvalidValue;
            const int lane = k++ % (BSB_AUX_STREAMS + 1);
            cudaStream_t s = conc && lane ? ms->aux[lane - 1] : st;
            const int32_t *r = ranges + kRangeInts * t;
            if (tile_ev) cudaEventRecord(tile_ev[2 * t], s);
            if (f16) {
                // the wide class is rare (very large h0): one block per SM drains it
                e = f16(Q, d_jobs, d_seq, order, r, counter + 3 * t, d_out, d_cells, n_sm, s);
                if (e == cudaSuccess) e = f(Q, d_jobs, d_seq, order, r + 2, counter + 3 * t + 1, d_out, d_cells, -n_sm, s);
            } else {
                e = f(Q, d_jobs, d_seq, order, r + 4, counter + 3 * t + 2, d_out, d_cells, n_sm, s);
            }
            if (e != cudaSuccess) return e;
            if (tile_ev) cudaEventRecord(tile_ev[2 * t + 1], s);
        }
        if (conc) {
            for (int a = 0; a < BSB_AUX_STREAMS; ++a) {
                cudaEventRecord(ms->join[a], ms->aux[a]);
                cudaStreamWaitEvent(st, ms->join[a], 0);
            }
        }
    }
    if (ev1) cudaEventRecord(ev1, st);
    return cudaSuccess;
}
