// int_probe.cu -- measured integer-pipe peaks used as the extension roofline.
//
// The extension DP is built from integer adds and maxima.  These probes run the
// same two operations, add then max, in 8 independent chains per thread on every
// SM, and report the achieved rate counting each add and each max as one
// operation -- the unit in which the extension's algorithmic work (14 integer
// operations per DP cell) is counted: on 32-bit values (the 32-bit cell kernels),
// and on two 16-bit values per register (__viaddmax_s16x2, the 16-bit cell
// kernels), where one instruction carries four operations.

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
        }
        k1 ^= a0 & 1;   // keeps the compiler from folding the chains: 2 instructions per 128 operations
    }
    const int r = a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7;
    if (r == 0x7fffffff) sink[0] = r;
}

__global__ void __launch_bounds__(256) int16x2_probe_kernel(int iters, unsigned k1, unsigned k2, int *sink)
{
    unsigned a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
    unsigned a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            a0 = __viaddmax_s16x2(a0, k1, k2); a1 = __viaddmax_s16x2(a1, k1, k2);
            a2 = __viaddmax_s16x2(a2, k1, k2); a3 = __viaddmax_s16x2(a3, k1, k2);
            a4 = __viaddmax_s16x2(a4, k1, k2); a5 = __viaddmax_s16x2(a5, k1, k2);
            a6 = __viaddmax_s16x2(a6, k1, k2); a7 = __viaddmax_s16x2(a7, k1, k2);
        }
        k1 ^= a0 & 1;   // as above: 2 instructions per 64 counted ones
    }
    const unsigned r = a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7;
    if (r == 0x7fffffffu) sink[0] = (int)r;
}

template <typename K>
int run_probe(bsb_ctx *ctx, K kernel, unsigned k1, unsigned k2, double ops_per_step, double *tops, double *ms_out)
{
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    if ((rc = bsb_ensure(ctx, &ctx->scratch, &ctx->scratch_bytes, 256, "probe scratch"))) return rc;
    const int blocks = ctx->n_sm * 8, threads = 256, iters = 4096;
    kernel<<<blocks, threads, 0, ctx->stream>>>(64, k1, k2, (int *)ctx->scratch);   // warm-up
    cudaEventRecord(ctx->ev0, ctx->stream);
    kernel<<<blocks, threads, 0, ctx->stream>>>(iters, k1, k2, (int *)ctx->scratch);
    cudaEventRecord(ctx->ev1, ctx->stream);
    if ((rc = bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "int probe"))) return rc;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    const double ops = (double)blocks * threads * iters * 8.0 * ops_per_step;
    *tops = ops / (ms * 1e-3) / 1e12;
    if (ms_out) *ms_out = ms;
    return 0;
}

}  // namespace

extern "C" int bsb_probe_int16x2_peak(bsb_ctx *ctx, double *tops, double *ms_out)
{
    if (!ctx || !tops) return BSB_EINVAL;
    // per inner step: 8 chains x 2 halves x (add + max) = 32 operations
    return run_probe(ctx, int16x2_probe_kernel, 0x00010001u, 0xfffbfffbu, 32.0, tops, ms_out);
}

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
    // per inner step: 8 chains x (add + max) = 16 operations (one xor and one and per 8 steps)
    const double ops = (double)blocks * threads * iters * 8.0 * 16.0;
    *tops = ops / (ms * 1e-3) / 1e12;
    if (ms_out) *ms_out = ms;
    return 0;
}
