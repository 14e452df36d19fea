// ksw_tiles_impl.cuh -- the persistent per-tile extension kernels and their launchers,
// instantiated once per shape by ksw_tiles_g{4,8,16,32}.cu: the 32-bit cell kernel for
// every shape, and the 16-bit two-columns-per-register kernel (ksw_group16.cuh) for the
// shapes with an even C.
#pragma once

#include "ksw_group16.cuh"
#include "ksw_tiles.cuh"

// Shapes up to 18 columns per lane are held to 128 registers (4 blocks = 16 warps per
// SM): measured on GB300, the extra warps hide the ALU dependency latency better than
// the registers they cost (a few bytes of spill at C >= 15), 3-18 % faster.  Wider
// 32-bit shapes keep their registers.
constexpr int ksw_min_blocks(int C) { return C <= 18 ? 4 : 1; }
// The 16-bit kernels hold E, H and M of their C2 = C/2 registers plus the C profile words:
// with 4 lanes per job, 4 blocks fit without spills up to C2 = 12 (128 registers), 3 up to
// C2 = 16 (168).
constexpr int ksw16_min_blocks(int C2, int G)
{
    return G != 4 ? ksw_min_blocks(2 * C2) : C2 <= 12 ? 4 : 3;
}

// range[0], range[1]: the jobs order[range[0] .. range[1]) this launch drains.
template <int C, int G>
__global__ void __launch_bounds__(kKswBlock, ksw_min_blocks(C))
ksw_tile_kernel(KswParams P, const bsb_ext_job_t *__restrict__ jobs, const uint8_t *__restrict__ seq,
                const int32_t *__restrict__ order, const int32_t *__restrict__ range, int *__restrict__ counter,
                bsb_ext_out_t *__restrict__ out, int64_t *__restrict__ cells)
{
    ksw_group_run<C, G>(P, jobs, seq, order, range[0], range[1], counter, out, cells);
}

template <int C2, int G>
__global__ void __launch_bounds__(kKswBlock, ksw16_min_blocks(C2, G))
ksw_tile16_kernel(KswParams P, const bsb_ext_job_t *__restrict__ jobs, const uint8_t *__restrict__ seq,
                  const int32_t *__restrict__ order, const int32_t *__restrict__ range, int *__restrict__ counter,
                  bsb_ext_out_t *__restrict__ out, int64_t *__restrict__ cells)
{
    ksw_group16_run<C2, G>(P, jobs, seq, order, range[0], range[1], counter, out, cells);
}

// One resident wave of blocks; the warps drain the range's queue.  n_sm < 0 asks for
// one block per SM (-n_sm blocks), for a range that is expected to be short.
template <typename K>
cudaError_t ksw_launch_wave(K kernel, int &blocks_per_sm, const KswParams &P, const bsb_ext_job_t *jobs,
                            const uint8_t *seq, const int32_t *order, const int32_t *range, int *counter,
                            bsb_ext_out_t *out, int64_t *cells, int n_sm, cudaStream_t st)
{
    if (!blocks_per_sm) {
        int b = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, kKswBlock, 0);
        if (e != cudaSuccess) return e;
        blocks_per_sm = b < 1 ? 1 : b;
    }
    const int blocks = n_sm < 0 ? -n_sm : n_sm * blocks_per_sm;
    kernel<<<blocks, kKswBlock, 0, st>>>(P, jobs, seq, order, range, counter, out, cells);
    return cudaGetLastError();
}

template <int C, int G>
cudaError_t ksw_tile_launch(const KswParams &P, const bsb_ext_job_t *jobs, const uint8_t *seq,
                            const int32_t *order, const int32_t *range, int *counter, bsb_ext_out_t *out,
                            int64_t *cells, int n_sm, cudaStream_t st)
{
    static int blocks_per_sm = 0;
    return ksw_launch_wave(ksw_tile_kernel<C, G>, blocks_per_sm, P, jobs, seq, order, range, counter, out, cells,
                           n_sm, st);
}

template <int C2, int G>
cudaError_t ksw_tile16_launch(const KswParams &P, const bsb_ext_job_t *jobs, const uint8_t *seq,
                              const int32_t *order, const int32_t *range, int *counter, bsb_ext_out_t *out,
                              int64_t *cells, int n_sm, cudaStream_t st)
{
    static int blocks_per_sm = 0;
    return ksw_launch_wave(ksw_tile16_kernel<C2, G>, blocks_per_sm, P, jobs, seq, order, range, counter, out,
                           cells, n_sm, st);
}
