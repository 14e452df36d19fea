// int_probe.cu -- measured integer-pipe peak used as the extension roofline.
//
// The extension DP is built from 32-bit integer adds and maxima.  This probe
// runs the same two operations, add then max, in 8 independent chains per
// thread on every SM, and reports the achieved rate counting each add and
// each max as one operation -- the unit in which the extension's algorithmic
// work (14 integer operations per DP cell) is counted.

#include "bsb_internal.cuh"

namespace {

__global__ void __launch_bounds__(256) int_probe_kernel(int iters, int k1, int k2, int *sink)
{
    int a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
    int a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            a0 = max(a0 + k1, k2); a1 = max(a1 + k1, k2); a2 = max(a2 + k1, k2); a3 = max(a3 + k1, k2);
            a4 = max(a4 + k1, k2); a5 = max(a5 + k1, k2); a6 = max(a6 + k1, k2); a7 = max(a7 + k1, k2);
            k1 ^= a0 & 1;   // keeps the compiler from folding the chains
        }
    }
    const int r = a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7;
    if (r == 0x7fffffff) sink[0] = r;
}

}  // namespace

extern "C" int bsb_probe_int_peak(bsb_ctx *ctx, double *tops, double *ms_out)
{
    if (!ctx || !tops) return BSB_EINVAL;
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    if ((rc = bsb_ensure(ctx, &ctx->scratch, &ctx->scratch_bytes, 256, "probe scratch"))) return rc;
    const int blocks = ctx->n_sm * 8, threads = 256, iters = 4096;
    int_probe_kernel<<<blocks, threads, 0, ctx->stream>>>(64, 1, -5, (int *)ctx->scratch);   // warm-up
    cudaEventRecord(ctx->ev0, ctx->stream);
    int_probe_kernel<<<blocks, threads, 0, ctx->stream>>>(iters, 1, -5, (int *)ctx->scratch);
    cudaEventRecord(ctx->ev1, ctx->stream);
    if ((rc = bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "int probe"))) return rc;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    // per inner step: 8 chains x (add + max) = 16 operations, plus one xor and one and
    const double ops = (double)blocks * threads * iters * 8.0 * 16.0;
    *tops = ops / (ms * 1e-3) / 1e12;
    if (ms_out) *ms_out = ms;
    return 0;
}
