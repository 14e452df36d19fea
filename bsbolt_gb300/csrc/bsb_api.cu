// bsb_api.cu -- extern "C" boundary of the sm_103a bisulfite seed/extend library.
//
// Owns the context (device, stream, events, growable device scratch) and the
// argument checks that turn the reference's assert()/err_fatal() exits into
// error codes.

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <new>
#include <thread>
#include <vector>

#include "bsb_internal.cuh"

int bsb_fail(bsb_ctx *ctx, int code, const char *fmt, ...)
{
    if (ctx) {
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->err = buf;
    }
    return code;
}

int bsb_cuda(bsb_ctx *ctx, cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return 0;
    if (e == cudaErrorMemoryAllocation)
        return bsb_fail(ctx, BSB_ENOMEM, "%s: %s", what, cudaGetErrorString(e));
    return bsb_fail(ctx, BSB_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

int bsb_ensure(bsb_ctx *ctx, void **buf, size_t *cur, size_t bytes, const char *what)
{
    if (*cur >= bytes && *buf) return 0;
    if (*buf) {
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return bsb_cuda(ctx, e, what);
        cudaFree(*buf);
        *buf = nullptr;
        *cur = 0;
    }
    size_t want = bytes + bytes / 4 + 4096;   // grow with headroom
    cudaError_t e = cudaMalloc(buf, want);
    if (e != cudaSuccess) {
        *buf = nullptr;
        return bsb_cuda(ctx, e, what);
    }
    *cur = want;
    return 0;
}

extern "C" {

const char *bsb_strerror(int code)
{
    switch (code) {
    case BSB_OK: return "ok";
    case BSB_EINVAL: return "invalid argument";
    case BSB_ECUDA: return "CUDA error";
    case BSB_ENOMEM: return "out of memory";
    case BSB_EIO: return "index I/O error";
    case BSB_ETIMEOUT: return "bounded device wait timed out";
    case BSB_ETOOLONG: return "sequence too long";
    case BSB_ENOINDEX: return "no index loaded";
    default: return "unknown error";
    }
}

int bsb_ctx_create(int device, bsb_ctx **out)
{
    if (!out) return BSB_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return BSB_ECUDA;
    if (device < 0 || device >= ndev) return BSB_EINVAL;
    bsb_ctx *ctx = new (std::nothrow) bsb_ctx();
    if (!ctx) return BSB_ENOMEM;
    ctx->device = device;
    memcpy(ctx->tile_map, ksw_default_tile_map(), BSB_TILE_MAP_LEN);
    ctx->map_tiles = ksw_map_tiles(ctx->tile_map);
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(device), "cudaSetDevice")) ||
        (rc = bsb_cuda(ctx, cudaDeviceGetAttribute(&ctx->n_sm, cudaDevAttrMultiProcessorCount, device), "sm count")) ||
        (rc = bsb_cuda(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "stream")) ||
        (rc = bsb_cuda(ctx, cudaEventCreate(&ctx->ev0), "event")) ||
        (rc = bsb_cuda(ctx, cudaEventCreate(&ctx->ev1), "event"))) {
        bsb_ctx_destroy(ctx);
        return rc;
    }
    bool ok = true;
    for (int t = 0; t < 2 * BSB_NUM_TILES && ok; ++t) ok = cudaEventCreate(&ctx->tile_ev[t]) == cudaSuccess;
    for (int t = 0; t < 4 * BSB_MAX_CHUNKS && ok; ++t)
        ok = cudaEventCreateWithFlags(&ctx->chunk_ev[t], (t & 3) < 2 ? cudaEventDisableTiming : cudaEventDefault) ==
             cudaSuccess;
    for (int t = 0; t <= BSB_ALIGN_STAGES && ok; ++t) ok = cudaEventCreate(&ctx->stage_ev[t]) == cudaSuccess;
    for (int a = 0; a < BSB_AUX_STREAMS && ok; ++a)
        ok = cudaStreamCreateWithFlags(&ctx->ms.aux[a], cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&ctx->ms.join[a], cudaEventDisableTiming) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&ctx->ms.fork, cudaEventDisableTiming) == cudaSuccess &&
         cudaStreamCreateWithFlags(&ctx->h2d, cudaStreamNonBlocking) == cudaSuccess &&
         cudaStreamCreateWithFlags(&ctx->d2h, cudaStreamNonBlocking) == cudaSuccess;
    if (!ok) {
        rc = bsb_cuda(ctx, cudaGetLastError(), "streams and events");
        bsb_ctx_destroy(ctx);
        return rc ? rc : BSB_ECUDA;
    }
    *out = ctx;
    return BSB_OK;
}

void bsb_ctx_destroy(bsb_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->d_in) cudaFree(ctx->d_in);
    if (ctx->d_out) cudaFree(ctx->d_out);
    if (ctx->seed_scratch) cudaFree(ctx->seed_scratch);
    if (ctx->arena0) cudaFree(ctx->arena0);
    if (ctx->arena1) cudaFree(ctx->arena1);
    if (ctx->arena2) cudaFree(ctx->arena2);
    if (ctx->flt_in) cudaFree(ctx->flt_in);
    if (ctx->flt_out) cudaFree(ctx->flt_out);
    if (ctx->flt_dev) cudaFree(ctx->flt_dev);
    if (ctx->rc_buf) cudaFree(ctx->rc_buf);
    if (ctx->d_tile_map) cudaFree(ctx->d_tile_map);
    bsb_index_release(ctx);
    for (cudaStream_t s : {ctx->h2d, ctx->d2h, ctx->ms.aux[0], ctx->ms.aux[1], ctx->ms.aux[2]})
        if (s) cudaStreamSynchronize(s);
    for (int t = 0; t < 2 * BSB_NUM_TILES; ++t)
        if (ctx->tile_ev[t]) cudaEventDestroy(ctx->tile_ev[t]);
    for (int t = 0; t < 4 * BSB_MAX_CHUNKS; ++t)
        if (ctx->chunk_ev[t]) cudaEventDestroy(ctx->chunk_ev[t]);
    for (int t = 0; t <= BSB_ALIGN_STAGES; ++t)
        if (ctx->stage_ev[t]) cudaEventDestroy(ctx->stage_ev[t]);
    for (int a = 0; a < BSB_AUX_STREAMS; ++a) {
        if (ctx->ms.aux[a]) cudaStreamDestroy(ctx->ms.aux[a]);
        if (ctx->ms.join[a]) cudaEventDestroy(ctx->ms.join[a]);
    }
    if (ctx->ms.fork) cudaEventDestroy(ctx->ms.fork);
    if (ctx->h2d) cudaStreamDestroy(ctx->h2d);
    if (ctx->d2h) cudaStreamDestroy(ctx->d2h);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char *bsb_last_error(const bsb_ctx *ctx)
{
    return ctx ? ctx->err.c_str() : "no context";
}

void *bsb_ctx_stream(bsb_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

float bsb_last_kernel_ms(const bsb_ctx *ctx) { return ctx ? ctx->last_kernel_ms : 0.f; }

}  // extern "C"

// Host batches of at least this many jobs are extended in BSB_MAX_CHUNKS pieces.
static const int64_t kChunkFrom = (int64_t)1 << 20;

static int check_param(bsb_ctx *ctx, const bsb_ext_param_t *param, KswParams *P)
{
    if (!param) return bsb_fail(ctx, BSB_EINVAL, "param is NULL");
    if (param->e_del < 1 || param->e_ins < 1)
        return bsb_fail(ctx, BSB_EINVAL, "gap extension penalties must be >= 1 (got %d, %d)",
                        param->e_del, param->e_ins);
    if (param->o_del < 0 || param->o_ins < 0)
        return bsb_fail(ctx, BSB_EINVAL, "gap open penalties must be >= 0");
    if (param->o_del > 65535 || param->o_ins > 65535 || param->e_del > 65535 || param->e_ins > 65535)
        return bsb_fail(ctx, BSB_EINVAL, "gap penalties must be <= 65535");
    memcpy(P->mat, param->mat, 25);
    P->o_del = param->o_del; P->e_del = param->e_del;
    P->o_ins = param->o_ins; P->e_ins = param->e_ins;
    P->zdrop = param->zdrop;
    int mx = 0;
    for (int i = 0; i < 25; ++i) mx = mx > param->mat[i] ? mx : param->mat[i];
    P->mat_max = mx;
    for (int i = 0; i < 25; ++i)
        if (param->mat[i] > 63 || param->mat[i] < -63)
            return bsb_fail(ctx, BSB_EINVAL, "scoring matrix entries must lie in [-63, 63]");
    return 0;
}

// Host-side validation of a job table (the kernel trusts what passes here).
// The precondition message for the first failing job of jobs[0..n) (numbered from first).
static int check_jobs(bsb_ctx *ctx, const bsb_ext_job_t *jobs, int64_t n, int64_t seq_bytes, int64_t first = 0)
{
    const int qmax = ksw_max_qlen();
    for (int64_t k = 0; k < n; ++k) {
        const bsb_ext_job_t &j = jobs[k];
        const int64_t i = first + k;
        if (j.qlen < 0 || j.tlen < 0 || j.w < 0 || j.flags != 0)
            return bsb_fail(ctx, BSB_EINVAL, "job %lld: negative length/band or nonzero flags", (long long)i);
        if (j.h0 <= 0 || j.h0 > (1 << 20))
            return bsb_fail(ctx, BSB_EINVAL, "job %lld: h0 must be in [1, 2^20] (ksw.c:385 asserts h0 > 0)",
                            (long long)i);
        if (j.qlen > qmax)
            return bsb_fail(ctx, BSB_ETOOLONG, "job %lld: qlen %d exceeds %d", (long long)i, j.qlen, qmax);
        if (j.qoff < 0 || j.toff < 0 || j.qoff + j.qlen > seq_bytes || j.toff + j.tlen > seq_bytes)
            return bsb_fail(ctx, BSB_EINVAL, "job %lld: sequence range outside the buffer", (long long)i);
        if ((int64_t)j.qlen + j.tlen > (1 << 30))
            return bsb_fail(ctx, BSB_ETOOLONG, "job %lld: sequence too long", (long long)i);
    }
    return 0;
}

// What the host entry needs from one stretch of jobs: the first job failing the
// preconditions (n if none), the shapes its query lengths map to, and the end of the
// sequence bytes it references.
struct JobScan {
    int64_t first_bad;
    uint64_t tiles;
    int64_t need;
};

static bool job_ok(const bsb_ext_job_t &j, int64_t seq_bytes, int qmax)
{
    return j.qlen >= 0 && j.tlen >= 0 && j.w >= 0 && j.flags == 0 && j.h0 > 0 && j.h0 <= (1 << 20) &&
           j.qlen <= qmax && j.qoff >= 0 && j.toff >= 0 && j.qoff + j.qlen <= seq_bytes &&
           j.toff + j.tlen <= seq_bytes && (int64_t)j.qlen + j.tlen <= (1 << 30);
}

static JobScan scan_jobs(const bsb_ext_job_t *jobs, int64_t lo, int64_t hi, int64_t seq_bytes,
                         const uint8_t *tile_map)
{
    const int qmax = ksw_max_qlen();
    JobScan r{hi, 0, 0};
    for (int64_t i = lo; i < hi; ++i) {
        const bsb_ext_job_t &j = jobs[i];
        if (!job_ok(j, seq_bytes, qmax)) {
            r.first_bad = i;
            break;
        }
        r.tiles |= 1ull << tile_map[j.qlen + 1];
        r.need = r.need > j.qoff + j.qlen ? r.need : j.qoff + j.qlen;
        r.need = r.need > j.toff + j.tlen ? r.need : j.toff + j.tlen;
    }
    return r;
}

// scan_jobs over pieces [k*per, (k+1)*per), host threads sharing the work for large
// batches (the scan is on the host entry's critical path before any device work).
static void scan_pieces(const bsb_ext_job_t *jobs, int64_t n, int64_t per, int nck, int64_t seq_bytes,
                        const uint8_t *tile_map, JobScan *piece)
{
    const int64_t kSlice = 1 << 16;
    const int64_t n_slices = (n + kSlice - 1) / kSlice;
    std::vector<JobScan> sl((size_t)n_slices);
    auto run = [&](int64_t a, int64_t b) {
        for (int64_t k = a; k < b; ++k)
            sl[(size_t)k] = scan_jobs(jobs, k * kSlice, std::min(n, (k + 1) * kSlice), seq_bytes, tile_map);
    };
    unsigned hw = std::thread::hardware_concurrency();
    int T = (int)std::min<int64_t>(n_slices, hw ? (int64_t)hw : 4);
    if (T > 16) T = 16;
    if (T <= 1) {
        run(0, n_slices);
    } else {
        std::vector<std::thread> th;
        for (int t = 0; t < T; ++t) th.emplace_back(run, n_slices * t / T, n_slices * (t + 1) / T);
        for (auto &x : th) x.join();
    }
    for (int k = 0; k < nck; ++k) piece[k] = JobScan{n, 0, 0};
    for (int64_t k = 0; k < n_slices; ++k) {        // a slice may straddle two pieces: split it
        const int64_t lo = k * kSlice, hi = std::min(n, lo + kSlice);
        const int a = (int)(lo / per), b = (int)((hi - 1) / per);
        if (a == b) {
            JobScan &p = piece[a];
            p.first_bad = std::min(p.first_bad, sl[(size_t)k].first_bad < hi ? sl[(size_t)k].first_bad : n);
            p.tiles |= sl[(size_t)k].tiles;
            p.need = std::max(p.need, sl[(size_t)k].need);
        } else {
            for (int c = a; c <= b; ++c) {
                const JobScan q = scan_jobs(jobs, std::max(lo, c * per), std::min(hi, (c + 1) * per), seq_bytes,
                                            tile_map);
                JobScan &p = piece[c];
                p.first_bad = std::min(p.first_bad, q.first_bad < std::min(hi, (c + 1) * per) ? q.first_bad : n);
                p.tiles |= q.tiles;
                p.need = std::max(p.need, q.need);
            }
        }
    }
}

// Device-buffer extension with the tile shapes `tiles` launched (every shape
// the context's map uses when the caller cannot tell which are needed).
static int extend_device(bsb_ctx *ctx, const bsb_ext_param_t *param, const bsb_ext_job_t *d_jobs,
                         int64_t n_jobs, const uint8_t *d_seq, int64_t seq_bytes, const int32_t *d_cost,
                         bsb_ext_out_t *d_out, int64_t *d_cells, uint64_t tiles, cudaEvent_t e0 = nullptr,
                         cudaEvent_t e1 = nullptr)
{
    if (!ctx) return BSB_EINVAL;
    KswParams P;
    int rc = check_param(ctx, param, &P);
    if (rc) return rc;
    if (n_jobs < 0 || n_jobs > (int64_t)0x7fffffff) return bsb_fail(ctx, BSB_EINVAL, "n_jobs out of range");
    if (n_jobs == 0) return 0;
    if (!d_jobs || !d_seq || !d_out) return bsb_fail(ctx, BSB_EINVAL, "NULL buffer");
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    if ((rc = bsb_ensure(ctx, &ctx->scratch, &ctx->scratch_bytes, ksw_scratch_bytes(n_jobs), "extension scratch")))
        return rc;
    cudaError_t e = ksw_launch(P, d_jobs, n_jobs, seq_bytes, d_seq, d_cost, ctx->d_tile_map, tiles, d_out, d_cells,
                               ctx->scratch, ctx->n_sm, ctx->stream, e0 ? e0 : ctx->ev0, e1 ? e1 : ctx->ev1,
                               ctx->tile_ev, &ctx->ms);
    ctx->pending_ksw = 1;
    ctx->last_tiles = tiles;
    return bsb_cuda(ctx, e, "extension launch");
}

extern "C" int bsb_extend_batch_device(bsb_ctx *ctx, const bsb_ext_param_t *param,
                                       const bsb_ext_job_t *d_jobs, int64_t n_jobs,
                                       const uint8_t *d_seq, int64_t seq_bytes,
                                       const int32_t *d_cost, bsb_ext_out_t *d_out, int64_t *d_cells)
{
    if (!ctx) return BSB_EINVAL;
    return extend_device(ctx, param, d_jobs, n_jobs, d_seq, seq_bytes, d_cost, d_out, d_cells, ctx->map_tiles);
}

extern "C" int bsb_tile_shapes(int32_t *G, int32_t *C, int max)
{
    for (int t = 0; t < BSB_NUM_TILES && t < max; ++t) {
        int g = 0, c = 0;
        ksw_tile_shape(t, &g, &c);
        if (G) G[t] = g;
        if (C) C[t] = c;
    }
    return BSB_NUM_TILES;
}

extern "C" int bsb_set_tile_map(bsb_ctx *ctx, const uint8_t *map, int n)
{
    if (!ctx) return BSB_EINVAL;
    if (!map) {
        memcpy(ctx->tile_map, ksw_default_tile_map(), BSB_TILE_MAP_LEN);
        ctx->map_tiles = ksw_map_tiles(ctx->tile_map);
        if (ctx->d_tile_map) {
            cudaSetDevice(ctx->device);
            cudaStreamSynchronize(ctx->stream);
            cudaFree(ctx->d_tile_map);
            ctx->d_tile_map = nullptr;
        }
        return 0;
    }
    if (n != BSB_TILE_MAP_LEN)
        return bsb_fail(ctx, BSB_EINVAL, "tile map must have %d entries (got %d)", BSB_TILE_MAP_LEN, n);
    for (int need = 1; need < BSB_TILE_MAP_LEN; ++need) {
        int g = 0, c = 0;
        if (ksw_tile_shape(map[need], &g, &c))
            return bsb_fail(ctx, BSB_EINVAL, "tile map entry %d names shape %d (of %d)", need, map[need], BSB_NUM_TILES);
        if (g * c < need)
            return bsb_fail(ctx, BSB_EINVAL, "tile map entry %d: shape %d (%d x %d) holds %d columns", need, map[need],
                            g, c, g * c);
    }
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    if (!ctx->d_tile_map &&
        (rc = bsb_cuda(ctx, cudaMalloc((void **)&ctx->d_tile_map, BSB_TILE_MAP_LEN), "tile map")))
        return rc;
    // batches already queued read the old map: the copy is ordered after them
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(ctx->d_tile_map, map, BSB_TILE_MAP_LEN, cudaMemcpyHostToDevice,
                                            ctx->stream), "tile map upload")) ||
        (rc = bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "tile map upload")))
        return rc;
    memcpy(ctx->tile_map, map, BSB_TILE_MAP_LEN);
    ctx->tile_map[0] = 0;
    ctx->map_tiles = ksw_map_tiles(ctx->tile_map);
    return 0;
}

extern "C" int bsb_last_tile_ms(const bsb_ctx *ctx, float *ms, int n)
{
    if (!ctx || !ms) return BSB_EINVAL;
    for (int t = 0; t < BSB_NUM_TILES && t < n; ++t) ms[t] = ctx->tile_ms[t];
    return 0;
}

extern "C" int bsb_get_tile_map(bsb_ctx *ctx, uint8_t *map, int n)
{
    if (!map || n < BSB_TILE_MAP_LEN) return ctx ? bsb_fail(ctx, BSB_EINVAL, "tile map buffer too small") : BSB_EINVAL;
    memcpy(map, ctx ? ctx->tile_map : ksw_default_tile_map(), BSB_TILE_MAP_LEN);
    return 0;
}

extern "C" int bsb_extend_batch(bsb_ctx *ctx, const bsb_ext_param_t *param, const bsb_ext_job_t *jobs,
                                int64_t n_jobs, const uint8_t *seq, int64_t seq_bytes, bsb_ext_out_t *out,
                                int64_t *cells_out)
{
    if (!ctx) return BSB_EINVAL;
    if (n_jobs < 0) return bsb_fail(ctx, BSB_EINVAL, "n_jobs < 0");
    if (n_jobs == 0) return 0;
    if (!jobs || !seq || !out) return bsb_fail(ctx, BSB_EINVAL, "NULL buffer");
    KswParams P;
    int rc = check_param(ctx, param, &P);
    if (rc) return rc;
    // Large batches are extended in pieces of consecutive jobs: piece k starts once the
    // sequence prefix its jobs reference and its job records are on the device (h2d
    // stream), and its tuples return (d2h stream) while piece k+1 runs.  Jobs laid out in
    // buffer order make that prefix grow piece by piece; any other layout is still
    // correct, it just overlaps less.
    const int64_t per = n_jobs >= kChunkFrom ? (n_jobs + BSB_MAX_CHUNKS - 1) / BSB_MAX_CHUNKS : n_jobs;
    const int nck = (int)((n_jobs + per - 1) / per);
    JobScan piece[BSB_MAX_CHUNKS];
    scan_pieces(jobs, n_jobs, per, nck, seq_bytes, ctx->tile_map, piece);
    for (int k = 0; k < nck; ++k)          // every job is checked before any device work
        if (piece[k].first_bad < n_jobs) return check_jobs(ctx, jobs + piece[k].first_bad, 1, seq_bytes,
                                                           piece[k].first_bad);
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;

    const size_t jb = sizeof(bsb_ext_job_t) * (size_t)n_jobs;
    const size_t sb = ((size_t)seq_bytes + 255) & ~(size_t)255;
    const size_t ob = sizeof(bsb_ext_out_t) * (size_t)n_jobs;
    const size_t cb = cells_out ? sizeof(int64_t) * (size_t)n_jobs : 0;
    if ((rc = bsb_ensure(ctx, &ctx->d_in, &ctx->d_in_bytes, jb + sb + 256, "input staging"))) return rc;
    if ((rc = bsb_ensure(ctx, &ctx->d_out, &ctx->d_out_bytes, ob + cb + 256, "output staging"))) return rc;
    char *din = (char *)ctx->d_in;
    uint8_t *d_seq = (uint8_t *)din;
    bsb_ext_job_t *d_jobs = (bsb_ext_job_t *)(din + sb);
    bsb_ext_out_t *d_out = (bsb_ext_out_t *)ctx->d_out;
    int64_t *d_cells = cells_out ? (int64_t *)((char *)ctx->d_out + ((ob + 255) & ~(size_t)255)) : nullptr;

    if ((rc = bsb_ensure(ctx, &ctx->scratch, &ctx->scratch_bytes, ksw_scratch_bytes(per), "extension scratch")))
        return rc;
    // the stream must not still read the staging buffers from an earlier call when h2d overwrites them
    if ((rc = bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "stream synchronize"))) return rc;
    int64_t done = 0;
    for (int k = 0; k < nck; ++k) {
        const int64_t lo = k * per, cnt = n_jobs - lo < per ? n_jobs - lo : per;
        const int64_t need = piece[k].need;
        const uint64_t tiles = piece[k].tiles;     // only the shapes these query lengths map to
        cudaEvent_t *ev = ctx->chunk_ev + 4 * k;      // in, out, start, end
        if (need > done &&
            (rc = bsb_cuda(ctx, cudaMemcpyAsync(d_seq + done, seq + done, need - done, cudaMemcpyHostToDevice, ctx->h2d),
                           "H2D seq")))
            return rc;
        done = need > done ? need : done;
        if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(d_jobs + lo, jobs + lo, sizeof(bsb_ext_job_t) * cnt,
                                                cudaMemcpyHostToDevice, ctx->h2d), "H2D jobs")) ||
            (rc = bsb_cuda(ctx, cudaEventRecord(ev[0], ctx->h2d), "event")) ||
            (rc = bsb_cuda(ctx, cudaStreamWaitEvent(ctx->stream, ev[0], 0), "event")))
            return rc;
        if ((rc = extend_device(ctx, param, d_jobs + lo, cnt, d_seq, seq_bytes, nullptr, d_out + lo,
                                d_cells ? d_cells + lo : nullptr, tiles, ev[2], ev[3])))
            return rc;
        if ((rc = bsb_cuda(ctx, cudaEventRecord(ev[1], ctx->stream), "event")) ||
            (rc = bsb_cuda(ctx, cudaStreamWaitEvent(ctx->d2h, ev[1], 0), "event")) ||
            (rc = bsb_cuda(ctx, cudaMemcpyAsync(out + lo, d_out + lo, sizeof(bsb_ext_out_t) * cnt,
                                                cudaMemcpyDeviceToHost, ctx->d2h), "D2H out")))
            return rc;
        if (cells_out && (rc = bsb_cuda(ctx, cudaMemcpyAsync(cells_out + lo, d_cells + lo, sizeof(int64_t) * cnt,
                                                             cudaMemcpyDeviceToHost, ctx->d2h), "D2H cells")))
            return rc;
    }
    ctx->n_chunks = nck;
    if ((rc = bsb_cuda(ctx, cudaStreamSynchronize(ctx->d2h), "D2H synchronize"))) return rc;
    return bsb_sync(ctx);
}

extern "C" int bsb_sync(bsb_ctx *ctx)
{
    if (!ctx) return BSB_EINVAL;
    int rc;
    if ((rc = bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "stream synchronize"))) return rc;
    if (ctx->pending_ksw) {
        ctx->pending_ksw = 0;
        if (ctx->n_chunks) {        // a host batch in pieces: the sum of the pieces' extension times
            ctx->last_kernel_ms = 0.f;
            for (int k = 0; k < ctx->n_chunks; ++k) {
                float m = 0.f;
                cudaEventElapsedTime(&m, ctx->chunk_ev[4 * k + 2], ctx->chunk_ev[4 * k + 3]);
                ctx->last_kernel_ms += m;
            }
            ctx->n_chunks = 0;
        } else {
            cudaEventElapsedTime(&ctx->last_kernel_ms, ctx->ev0, ctx->ev1);
        }
        for (int t = 0; t < BSB_NUM_TILES; ++t) {
            ctx->tile_ms[t] = 0.f;
            if (ctx->last_tiles >> t & 1) cudaEventElapsedTime(&ctx->tile_ms[t], ctx->tile_ev[2 * t], ctx->tile_ev[2 * t + 1]);
        }
        int rej = 0;
        if ((rc = bsb_cuda(ctx, cudaMemcpy(&rej, ksw_rejected_counter(ctx->scratch), sizeof(int),
                                           cudaMemcpyDeviceToHost), "rejected-job counter")))
            return rc;
        if (rej) return bsb_fail(ctx, BSB_EINVAL, "%d extension jobs failed the preconditions and were skipped", rej);
    }
    return 0;
}
