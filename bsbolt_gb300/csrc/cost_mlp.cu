// cost_mlp.cu -- learned cost model for the extension scheduler.
//
// A 2 x 64 MLP predicts log(1 + DP cells) of a ksw_extend2 job from eight
// cheap features.  Its only use is the issue order of the persistent
// extension kernels (bsb_extend_batch_device's cost key): it never changes a
// result.  Weights are BF16 (the copy the forward pass reads), with FP32
// master weights and Adam moments for training; every product is
// accumulated in FP32.  The kernels are plain CUDA -- the model is far too
// small for the tensor cores to matter (8 -> 64 -> 64 -> 1 per job).
//
// Features (all O(1) per job except two 16-base scans):
//   f0 qlen/256   f1 tlen/512   f2 h0/128   f3 min(w, qlen)/256
//   f4 G fraction of the query (the converted alphabet's rare base)
//   f5 N fraction of query and target
//   f6 identity of the first 16 query/target bases (low -> early z-drop / zero row)
//   f7 log2(1 + plain bound qlen x min(tlen, qlen+w)) / 20

#include <cuda_bf16.h>

#include "bsb_internal.cuh"

namespace {

constexpr int F = BSB_MLP_FEATURES;
constexpr int H = BSB_MLP_HIDDEN;

__global__ void features_kernel(const bsb_ext_job_t *__restrict__ jobs, int64_t n, const uint8_t *__restrict__ seq,
                                int64_t seq_bytes, float *__restrict__ feat)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const bsb_ext_job_t j = jobs[i];
        float *f = feat + i * F;
        const bool ok = j.qlen >= 0 && j.tlen >= 0 && j.qoff >= 0 && j.toff >= 0 && j.qoff + j.qlen <= seq_bytes &&
                        j.toff + j.tlen <= seq_bytes;
        if (!ok) {
            for (int k = 0; k < F; ++k) f[k] = 0.f;
            continue;
        }
        const uint8_t *q = seq + j.qoff, *t = seq + j.toff;
        const int qs = j.qlen < 64 ? j.qlen : 64;       // composition from the first 64 bases
        int g = 0, nn = 0, id = 0;
        for (int k = 0; k < qs; ++k) {
            const int b = q[k];
            g += b == 2;
            nn += b > 3;
        }
        const int ts = j.tlen < 64 ? j.tlen : 64;
        for (int k = 0; k < ts; ++k) nn += t[k] > 3;
        const int m = min(16, min(j.qlen, j.tlen));
        for (int k = 0; k < m; ++k) id += q[k] == t[k] && q[k] < 4;
        const long long span = min((long long)j.tlen, (long long)j.qlen + j.w);
        const double bound = (double)j.qlen * (double)max(span, 0LL);
        f[0] = j.qlen / 256.f;
        f[1] = j.tlen / 512.f;
        f[2] = j.h0 / 128.f;
        f[3] = min(j.w, j.qlen) / 256.f;
        f[4] = qs ? (float)g / qs : 0.f;
        f[5] = (qs + ts) ? (float)nn / (qs + ts) : 0.f;
        f[6] = m ? (float)id / m : 0.f;
        f[7] = (float)(log2(1.0 + bound) / 20.0);
    }
}

__device__ __forceinline__ float bf(uint16_t u) { return __bfloat162float(__ushort_as_bfloat16(u)); }
__device__ __forceinline__ uint16_t to_bf(float x) { return __bfloat16_as_ushort(__float2bfloat16(x)); }

// Forward pass, one thread per job; the BF16 weights sit in shared memory.
// h1 = relu(W1 x + b1), h2 = relu(W2 h1 + b2), y = w3 . h2 + b3.
__global__ void __launch_bounds__(256) mlp_forward_kernel(const bsb_mlp_weights_t *__restrict__ W, const float *__restrict__ feat,
                                                          int64_t n, float *__restrict__ pred, int32_t *__restrict__ key)
{
    __shared__ float w1[H * F], w2[H * H], w3[H], b1[H], b2[H];
    __shared__ float b3;
    for (int k = threadIdx.x; k < H * F; k += blockDim.x) w1[k] = bf(W->w1[k]);
    for (int k = threadIdx.x; k < H * H; k += blockDim.x) w2[k] = bf(W->w2[k]);
    for (int k = threadIdx.x; k < H; k += blockDim.x) { w3[k] = bf(W->w3[k]); b1[k] = W->b1[k]; b2[k] = W->b2[k]; }
    if (threadIdx.x == 0) b3 = W->b3;
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float x[F], h1[H];
        for (int k = 0; k < F; ++k) x[k] = feat[i * F + k];
        for (int o = 0; o < H; ++o) {
            float a = b1[o];
            for (int k = 0; k < F; ++k) a = fmaf(w1[o * F + k], x[k], a);
            h1[o] = a > 0.f ? a : 0.f;
        }
        float y = b3;
        for (int o = 0; o < H; ++o) {
            float a = b2[o];
            for (int k = 0; k < H; ++k) a = fmaf(w2[o * H + k], h1[k], a);
            a = a > 0.f ? a : 0.f;
            y = fmaf(w3[o], a, y);
        }
        if (pred) pred[i] = y;
        if (key) {
            // cost key for the scheduler: predicted cells, clamped to int32
            const float c = expf(fminf(fmaxf(y, 0.f), 21.f)) - 1.f;
            key[i] = (int32_t)fminf(c, 2.0e9f);
        }
    }
}

// Backward, step 1 (one thread per sample): activations and the per-sample
// error signals of the loss mean((y - target)^2).  act row layout:
// h1[H] | d2[H] (dL/d pre-activation of layer 2) | d1[H] (layer 1) | dy.
constexpr int kActRow = 3 * H + 1;

__global__ void __launch_bounds__(128) mlp_signals_kernel(const bsb_mlp_weights_t *__restrict__ W, const float *__restrict__ feat,
                                                          const float *__restrict__ target, int n, float *__restrict__ act,
                                                          float *__restrict__ sq_err)
{
    __shared__ float w1[H * F], w2[H * H], w3[H], b1[H], b2[H];
    for (int k = threadIdx.x; k < H * F; k += blockDim.x) w1[k] = bf(W->w1[k]);
    for (int k = threadIdx.x; k < H * H; k += blockDim.x) w2[k] = bf(W->w2[k]);
    for (int k = threadIdx.x; k < H; k += blockDim.x) { w3[k] = bf(W->w3[k]); b1[k] = W->b1[k]; b2[k] = W->b2[k]; }
    __syncthreads();
    const float inv_n = 1.f / (float)n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float x[F], h1[H], d2[H];
        for (int k = 0; k < F; ++k) x[k] = feat[(int64_t)i * F + k];
        for (int o = 0; o < H; ++o) {
            float a = b1[o];
            for (int k = 0; k < F; ++k) a = fmaf(w1[o * F + k], x[k], a);
            h1[o] = a > 0.f ? a : 0.f;
        }
        float y = W->b3;
        for (int o = 0; o < H; ++o) {
            float a = b2[o];
            for (int k = 0; k < H; ++k) a = fmaf(w2[o * H + k], h1[k], a);
            d2[o] = a;                                   // pre-activation, turned into a signal below
            y = fmaf(w3[o], a > 0.f ? a : 0.f, y);
        }
        const float r = y - target[i];
        sq_err[i] = r * r;
        const float dy = 2.f * r * inv_n;
        float *row = act + (int64_t)i * kActRow;
        for (int o = 0; o < H; ++o) {
            row[o] = h1[o];
            const float pre = d2[o];
            d2[o] = pre > 0.f ? dy * w3[o] : 0.f;
            row[H + o] = d2[o];
        }
        for (int k = 0; k < H; ++k) {
            float s = 0.f;
            for (int o = 0; o < H; ++o) s = fmaf(d2[o], w2[o * H + k], s);
            row[2 * H + k] = h1[k] > 0.f ? s : 0.f;
        }
        row[3 * H] = dy;
    }
}

// Backward, step 2: one thread per parameter sums its gradient over the batch
// in sample order (deterministic, no atomics).  Parameter layout:
// w1[H*F] | w2[H*H] | w3[H] | b1[H] | b2[H] | b3 ; grad[BSB_MLP_PARAMS] = mean loss.
__global__ void mlp_param_grad_kernel(const float *__restrict__ feat, const float *__restrict__ act, int n,
                                      const float *__restrict__ sq_err, float *__restrict__ grad)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > BSB_MLP_PARAMS) return;
    float s = 0.f;
    if (p == BSB_MLP_PARAMS) {                       // the loss itself
        for (int i = 0; i < n; ++i) s += sq_err[i];
        grad[p] = s / (float)n;
        return;
    }
    if (p < H * F) {                                 // dW1[o][c] = d1[o] * x[c]
        const int o = p / F, c = p % F;
        for (int i = 0; i < n; ++i) s = fmaf(act[(int64_t)i * kActRow + 2 * H + o], feat[(int64_t)i * F + c], s);
    } else if (p < H * F + H * H) {                  // dW2[o][k] = d2[o] * h1[k]
        const int q = p - H * F, o = q / H, k = q % H;
        for (int i = 0; i < n; ++i) {
            const float *row = act + (int64_t)i * kActRow;
            s = fmaf(row[H + o], row[k], s);
        }
    } else if (p < H * F + H * H + H) {              // dw3: written by mlp_w3_grad_kernel
        return;
    } else if (p < H * F + H * H + 2 * H) {          // db1[o] = d1[o]
        const int o = p - H * F - H * H - H;
        for (int i = 0; i < n; ++i) s += act[(int64_t)i * kActRow + 2 * H + o];
    } else if (p < H * F + H * H + 3 * H) {          // db2[o] = d2[o]
        const int o = p - H * F - H * H - 2 * H;
        for (int i = 0; i < n; ++i) s += act[(int64_t)i * kActRow + H + o];
    } else {                                         // db3 = dy
        for (int i = 0; i < n; ++i) s += act[(int64_t)i * kActRow + 3 * H];
    }
    grad[p] = s;
}

// dw3[o] = sum_i dy_i * relu(W2 h1_i + b2)[o]; h2 is not kept, so it is
// recomputed here from h1 (one thread per output unit, samples in order).
__global__ void mlp_w3_grad_kernel(const bsb_mlp_weights_t *__restrict__ W, const float *__restrict__ act, int n,
                                   float *__restrict__ grad)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= H) return;
    float w2r[H];
    for (int k = 0; k < H; ++k) w2r[k] = bf(W->w2[o * H + k]);
    const float b2o = W->b2[o];
    float s = 0.f;
    for (int i = 0; i < n; ++i) {
        const float *row = act + (int64_t)i * kActRow;
        float a = b2o;
        for (int k = 0; k < H; ++k) a = fmaf(w2r[k], row[k], a);
        s = fmaf(row[3 * H], a > 0.f ? a : 0.f, s);
    }
    grad[H * F + H * H + o] = s;
}

// Adam on the FP32 master weights, then the BF16 copy the forward pass reads.
__global__ void adam_kernel(bsb_mlp_weights_t *__restrict__ W, float *__restrict__ master, float *__restrict__ m,
                            float *__restrict__ v, const float *__restrict__ grad, float lr, float b1p, float b2p)
{
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= BSB_MLP_PARAMS) return;
    const float g = grad[k];
    m[k] = beta1 * m[k] + (1.f - beta1) * g;
    v[k] = beta2 * v[k] + (1.f - beta2) * g * g;
    const float mh = m[k] / (1.f - b1p), vh = v[k] / (1.f - b2p);
    const float p = master[k] - lr * mh / (sqrtf(vh) + eps);
    master[k] = p;
    if (k < H * F) W->w1[k] = to_bf(p);
    else if (k < H * F + H * H) W->w2[k - H * F] = to_bf(p);
    else if (k < H * F + H * H + H) W->w3[k - H * F - H * H] = to_bf(p);
    else if (k < H * F + H * H + 2 * H) W->b1[k - H * F - H * H - H] = p;
    else if (k < H * F + H * H + 3 * H) W->b2[k - H * F - H * H - 2 * H] = p;
    else W->b3 = p;
}

}  // namespace

extern "C" int bsb_cost_features(bsb_ctx *ctx, const bsb_ext_job_t *d_jobs, int64_t n, const uint8_t *d_seq,
                                 int64_t seq_bytes, float *d_feat)
{
    if (!ctx || n < 0 || (n > 0 && (!d_jobs || !d_seq || !d_feat))) return BSB_EINVAL;
    if (n == 0) return 0;
    const int64_t want = (n + 255) / 256;
    const int blocks = (int)(want < (int64_t)ctx->n_sm * 16 ? want : (int64_t)ctx->n_sm * 16);
    features_kernel<<<blocks, 256, 0, ctx->stream>>>(d_jobs, n, d_seq, seq_bytes, d_feat);
    return bsb_cuda(ctx, cudaGetLastError(), "features launch");
}

extern "C" int bsb_mlp_forward(bsb_ctx *ctx, const bsb_mlp_weights_t *d_w, const float *d_feat, int64_t n,
                               float *d_pred, int32_t *d_key)
{
    if (!ctx || !d_w || n < 0 || (n > 0 && !d_feat)) return BSB_EINVAL;
    if (n == 0) return 0;
    const int64_t want = (n + 255) / 256;
    const int blocks = (int)(want < (int64_t)ctx->n_sm * 8 ? want : (int64_t)ctx->n_sm * 8);
    mlp_forward_kernel<<<blocks, 256, 0, ctx->stream>>>(d_w, d_feat, n, d_pred, d_key);
    return bsb_cuda(ctx, cudaGetLastError(), "MLP forward launch");
}

extern "C" int bsb_mlp_backward(bsb_ctx *ctx, const bsb_mlp_weights_t *d_w, const float *d_feat, const float *d_target,
                                int32_t n, float *d_grad)
{
    if (!ctx || !d_w || !d_feat || !d_target || !d_grad || n <= 0) return BSB_EINVAL;
    int rc;
    const size_t act_b = sizeof(float) * ((size_t)n * kActRow + (size_t)n) + 256;
    if ((rc = bsb_ensure(ctx, &ctx->arena2, &ctx->arena2_bytes, act_b, "MLP activations"))) return rc;
    float *act = (float *)ctx->arena2, *sq = act + (size_t)n * kActRow;
    const int blocks = (n + 127) / 128 < ctx->n_sm * 4 ? (n + 127) / 128 : ctx->n_sm * 4;
    mlp_signals_kernel<<<blocks, 128, 0, ctx->stream>>>(d_w, d_feat, d_target, n, act, sq);
    mlp_param_grad_kernel<<<(BSB_MLP_PARAMS + 1 + 127) / 128, 128, 0, ctx->stream>>>(d_feat, act, n, sq, d_grad);
    mlp_w3_grad_kernel<<<1, H, 0, ctx->stream>>>(d_w, act, n, d_grad);
    return bsb_cuda(ctx, cudaGetLastError(), "MLP backward launch");
}

extern "C" int bsb_mlp_adam(bsb_ctx *ctx, bsb_mlp_weights_t *d_w, float *d_master, float *d_m, float *d_v,
                            const float *d_grad, float lr, int32_t step)
{
    if (!ctx || !d_w || !d_master || !d_m || !d_v || !d_grad || step < 1) return BSB_EINVAL;
    const float b1p = powf(0.9f, (float)step), b2p = powf(0.999f, (float)step);
    adam_kernel<<<(BSB_MLP_PARAMS + 255) / 256, 256, 0, ctx->stream>>>(d_w, d_master, d_m, d_v, d_grad, lr, b1p, b2p);
    return bsb_cuda(ctx, cudaGetLastError(), "Adam launch");
}
