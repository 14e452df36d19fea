// ksw_tiles_impl.cuh -- the persistent per-tile extension kernel and its launcher,
// instantiated once per shape by ksw_tiles_g{4,8,16,32}.cu.
#pragma once

#include "ksw_group.cuh"
#include "ksw_tiles.cuh"

// Shapes up to 18 columns per lane are held to 128 registers (4 blocks = 16 warps per
// SM): measured on GB300, the extra warps hide the ALU dependency latency better than
// the registers they cost (a few bytes of spill at C >= 15), 3-18 % faster.  Wider
// shapes keep their registers.
constexpr int ksw_min_blocks(int C) { return C <= 18 ? 4 : 1; }

template <int C, int G>
__global__ void __launch_bounds__(kKswBlock, ksw_min_blocks(C))
ksw_tile_kernel(KswParams P, const bsb_ext_job_t *__restrict__ jobs, const uint8_t *__restrict__ seq,
                const int32_t *__restrict__ order, const int32_t *__restrict__ bin_start, int bin,
                int *__restrict__ counter, bsb_ext_out_t *__restrict__ out, int64_t *__restrict__ cells)
{
    ksw_group_run<C, G>(P, jobs, seq, order, bin_start[bin], bin_start[bin + 1], counter + bin, out, cells);
}

// One resident wave of blocks; the warps drain the bin's queue.
template <int C, int G>
cudaError_t ksw_tile_launch(const KswParams &P, const bsb_ext_job_t *jobs, const uint8_t *seq,
                            const int32_t *order, const int32_t *bin_start, int bin, int *counter,
                            bsb_ext_out_t *out, int64_t *cells, int n_sm, cudaStream_t st)
{
    static int blocks_per_sm = 0;
    if (!blocks_per_sm) {
        int b = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ksw_tile_kernel<C, G>, kKswBlock, 0);
        if (e != cudaSuccess) return e;
        blocks_per_sm = b < 1 ? 1 : b;
    }
    ksw_tile_kernel<C, G><<<n_sm * blocks_per_sm, kKswBlock, 0, st>>>(P, jobs, seq, order, bin_start, bin, counter,
                                                                        out, cells);
    return cudaGetLastError();
}
