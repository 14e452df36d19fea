// ksw_noalloc.cu -- the batched extension with no device allocation at all.
//
// Who needs it: a caller that may not call cudaMalloc -- for instance code
// running inside a host application whose memory manager owns the whole
// device, or code on a path where the implicit device synchronisation of
// cudaMalloc/cudaFree is not allowed.  bsb_extend_batch_device still needs
// the context's growable scratch (issue order, bin counters); this entry
// point takes that scratch from one fixed array in the library's device
// memory instead.  The caller passes every input and output buffer.
//
// The array holds the scheduling scratch for up to BSB_NOALLOC_MAX_JOBS
// jobs (about 2 MiB) and lives on every GPU that loads the library until the
// process exits.  Every call shares it and it keeps the last call's
// contents; the launch clears the counters that must start at zero.  Two
// calls whose work overlaps on the GPU (different streams, or different
// host threads on one device) race on it: order them on one stream.

#include <mutex>

#include "bsb_internal.cuh"

namespace {

constexpr size_t kStaticBytes = 65536 + sizeof(int32_t) * 2 * (size_t)BSB_NOALLOC_MAX_JOBS + 256;

__device__ __align__(256) unsigned char g_ext_scratch[kStaticBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void *g_scratch_addr[kMaxDevices];   // device address of g_ext_scratch, per device
int g_n_sm[kMaxDevices];

// Per-device set-up, on the first call with that device current: the host
// symbol g_ext_scratch is only a stand-in, the kernels need its device address.
int setup_device(int dev, void **addr, int *n_sm)
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_ext_scratch) != cudaSuccess || !p) return BSB_ECUDA;
        int sm = 0;
        if (cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sm <= 0)
            return BSB_ECUDA;
        g_n_sm[dev] = sm;
        g_scratch_addr[dev] = p;
    }
    *addr = g_scratch_addr[dev];
    *n_sm = g_n_sm[dev];
    return 0;
}

}  // namespace

extern "C" int bsb_extend_batch_noalloc(const bsb_ext_param_t *param, const bsb_ext_job_t *d_jobs, int64_t n_jobs,
                                        const uint8_t *d_seq, int64_t seq_bytes, bsb_ext_out_t *d_out,
                                        int64_t *d_cells, void *stream)
{
    if (!param || n_jobs < 0) return BSB_EINVAL;
    if (n_jobs > BSB_NOALLOC_MAX_JOBS) return BSB_ECAPACITY;
    if (n_jobs > 0 && (!d_jobs || !d_seq || !d_out)) return BSB_EINVAL;
    if (param->e_del < 1 || param->e_ins < 1 || param->o_del < 0 || param->o_ins < 0 || param->o_del > 65535 ||
        param->o_ins > 65535 || param->e_del > 65535 || param->e_ins > 65535)
        return BSB_EINVAL;
    KswParams P;
    int mx = 0;
    for (int i = 0; i < 25; ++i) {
        if (param->mat[i] > 63 || param->mat[i] < -63) return BSB_EINVAL;
        P.mat[i] = param->mat[i];
        mx = mx > param->mat[i] ? mx : param->mat[i];
    }
    P.mat_max = mx;
    P.o_del = param->o_del; P.e_del = param->e_del;
    P.o_ins = param->o_ins; P.e_ins = param->e_ins;
    P.zdrop = param->zdrop;
    if (ksw_scratch_bytes(n_jobs) > kStaticBytes) return BSB_ECAPACITY;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return BSB_ECUDA;
    void *scratch = nullptr;
    int n_sm = 0;
    int rc = setup_device(dev, &scratch, &n_sm);    // also for an empty batch: a warm-up call sets up
    if (rc) return rc;
    if (n_jobs == 0) return 0;
    static const uint64_t tiles = ksw_map_tiles(ksw_default_tile_map());
    cudaError_t e = ksw_launch(P, d_jobs, n_jobs, seq_bytes, d_seq, nullptr, nullptr, tiles, d_out, d_cells, scratch,
                               n_sm, (cudaStream_t)stream, nullptr, nullptr);
    return e == cudaSuccess ? 0 : BSB_ECUDA;
}
