// sw_pack16b.cu -- word-lane (ksw_i16) instances of the packed ksw_align2 passes (sw_pack.cuh)
// for queries of 17..40 segments of 8 lanes, four threads per job.  The word-lane range is split
// over two translation units so that they compile side by side.

#include "sw_pack.cuh"

namespace bsbsw {

cudaError_t sw_pack16_run_hi(bool rev, const PackParams &S, const bsb_sw_job_t *jobs, const uint8_t *seq,
                             const int32_t *list, int n, const int64_t *boff, int2 *bscratch, bsb_kswr_t *out,
                             uint8_t *rsl, int *ctr, int q, int n_sm, cudaStream_t st)
{
    return sw_pack_run<8, 17, 40, kPackMaxSeg16>(rev, S, jobs, seq, list, n, boff, bscratch, out, rsl, ctr, q, n_sm,
                                                  st);
}

}  // namespace bsbsw
