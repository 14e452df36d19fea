// bsb_index.cu -- device-resident FM-index and the seeding / SA-lookup entry points.
//
// The index arrays are taken once per context in the reference's own layout
// (64-byte occurrence blocks, uint64 sampled SA, 2-bit pac), so the BWA driver
// can hand over what bwa_idx_load already read (bwa.c:363-524) or the library
// can read the files itself (bwt_restore_bwt / bwt_restore_sa, bwt.c:420-457).
// On the device the occurrence array is re-cut into 32-symbol sectors
// (fm_index.cuh); the SA and pac stay as they are.

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "bsb_internal.cuh"
#include "fm_index.cuh"
#include "scan.cuh"

size_t seed_scratch_bytes(int n_threads, int max_len);
size_t seed_padded_entries(int64_t total_bases, int n_reads, int mult);
size_t seed_queue_entries(int64_t total_bases, int n_reads, int mult);
int seed_threads(int n_sm, int max_len, int n_reads, uint64_t seq_len);
cudaError_t seed_launch(const DevFM &F, int min_seed_len, float split_factor, int split_width, int max_mem_intv,
                        int n_reads, const uint8_t *d_seqs, const int64_t *d_offs, int max_len,
                        void *d_padded, int *d_count, int64_t *d_out_off, void *d_out,
                        void *d_lists, int *d_ctrl, void *d_queue, int64_t queue_cap, int *d_tot,
                        int64_t *d_scan_tmp, int mult, int n_sm, cudaStream_t st);
cudaError_t sa_launch(const DevFM &F, const uint64_t *d_rows, int64_t n, uint64_t *d_pos, int n_sm, cudaStream_t st);
cudaError_t sa_full_build(const DevFM &F, int64_t n_sa, uint64_t *full, int *failed, int n_sm, cudaStream_t st);

void bsb_index_release(bsb_ctx *ctx)
{
    if (ctx->idx_bwt) cudaFree(ctx->idx_bwt);
    if (ctx->idx_sb) cudaFree(ctx->idx_sb);
    ctx->idx_sb = nullptr;
    if (ctx->idx_sa) cudaFree(ctx->idx_sa);
    if (ctx->idx_pac) cudaFree(ctx->idx_pac);
    if (ctx->idx_sa_full) cudaFree(ctx->idx_sa_full);
    ctx->idx_sa_full = nullptr;
    if (ctx->idx_opac) cudaFree(ctx->idx_opac);
    ctx->idx_opac = nullptr;
    if (ctx->idx_ann_off) cudaFree(ctx->idx_ann_off);
    if (ctx->idx_ann_len) cudaFree(ctx->idx_ann_len);
    ctx->idx_bwt = ctx->idx_sa = ctx->idx_pac = ctx->idx_ann_off = ctx->idx_ann_len = nullptr;
    ctx->n_seqs = 0;
    ctx->has_index = 0;
}

static DevFM dev_fm(const bsb_ctx *ctx)
{
    DevFM F;
    F.blk = (const uint4 *)ctx->idx_bwt;
    F.sb = (const uint64_t *)ctx->idx_sb;
    F.sym64 = ctx->idx_sym64;
    F.sa = (const uint64_t *)ctx->idx_sa;
    F.sa_full = (const uint64_t *)ctx->idx_sa_full;
    F.primary = ctx->primary;
    F.seq_len = ctx->seq_len;
    for (int i = 0; i < 5; ++i) F.L2[i] = ctx->L2[i];
    int sh = 0;
    while ((1 << sh) < ctx->sa_intv) ++sh;
    F.sa_shift = sh;
    return F;
}

// The full suffix array, resident in HBM (8 bytes per row: 3.2 GB for a 100 Mb
// bisulfite reference), turns every bwt_sa into one load.  Built from the sampled one
// on the device; when it does not fit, bwt_sa keeps its LF walk.
static int build_sa_full(bsb_ctx *ctx)
{
    if (ctx->idx_sa_full) return 0;
    void *full = nullptr;
    int *failed = nullptr;
    if (cudaMalloc(&full, 8 * (ctx->seq_len + 1)) == cudaSuccess && cudaMalloc((void **)&failed, sizeof(int)) == cudaSuccess) {
        int h_failed = 1;
        if (cudaMemsetAsync(failed, 0, sizeof(int), ctx->stream) == cudaSuccess &&
            sa_full_build(dev_fm(ctx), (int64_t)ctx->n_sa, (uint64_t *)full, failed, ctx->n_sm, ctx->stream) == cudaSuccess &&
            cudaMemcpyAsync(&h_failed, failed, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream) == cudaSuccess &&
            cudaStreamSynchronize(ctx->stream) == cudaSuccess && !h_failed) {
            ctx->idx_sa_full = full;
            full = nullptr;
        }
    }
    if (full) cudaFree(full);
    if (failed) cudaFree(failed);
    cudaGetLastError();           // an allocation that did not fit is not an error
    return bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "full suffix array");
}

extern "C" int bsb_index_full_sa(bsb_ctx *ctx, int enable)
{
    if (!ctx) return BSB_EINVAL;
    if (!ctx->has_index) return bsb_fail(ctx, BSB_ENOINDEX, "no index loaded");
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice")) ||
        (rc = bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "stream synchronize")))
        return rc;
    if (!enable) {
        if (ctx->idx_sa_full) cudaFree(ctx->idx_sa_full);
        ctx->idx_sa_full = nullptr;
        return 0;
    }
    if ((rc = build_sa_full(ctx))) return rc;
    return ctx->idx_sa_full ? 0 : bsb_fail(ctx, BSB_ENOMEM, "the full suffix array does not fit in device memory");
}

// Re-cuts the reference's occurrence array (64-byte blocks of 128 symbols: four uint64
// counts, eight symbol words) into the 32-byte sectors occ_at reads; one thread per sector.
__global__ void occ_sectors_kernel(const uint32_t *__restrict__ ref, uint64_t n_sectors, uint4 *__restrict__ out)
{
    const uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (s >= n_sectors) return;
    const uint32_t *b = ref + (s >> 2) * 16;
    const int q = (int)(s & 3);
    uint32_t a = 0, c = 0, g = 0;
    for (int w = 0; w < 2 * q; ++w) word_counts(b[8 + w], 16, a, c, g);
    const uint64_t ca = ((uint64_t)b[1] << 32 | b[0]) + a;
    const uint64_t cc = ((uint64_t)b[3] << 32 | b[2]) + c;
    const uint64_t cg = ((uint64_t)b[5] << 32 | b[4]) + g;
    out[2 * s] = make_uint4((uint32_t)ca, (uint32_t)(ca >> 32), (uint32_t)cc, (uint32_t)(cc >> 32));
    out[2 * s + 1] = make_uint4((uint32_t)cg, (uint32_t)(cg >> 32), b[8 + 2 * q], b[9 + 2 * q]);
}

// The same re-cut into 64-symbol sectors: counts relative to the sector's 2^32-row
// superblock (whose block starts at word ((s >> 26) << 25) * 16), four symbol words.
__global__ void occ_sectors64_kernel(const uint32_t *__restrict__ ref, uint64_t n_sectors, uint4 *__restrict__ out)
{
    const uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (s >= n_sectors) return;
    const uint32_t *b = ref + (s >> 1) * 16;
    const uint32_t *sbk = ref + ((s >> 26) << 25) * 16;
    const int h = (int)(s & 1);
    uint32_t a = 0, c = 0, g = 0;
    for (int w = 0; w < 4 * h; ++w) word_counts(b[8 + w], 16, a, c, g);
    const uint64_t ca = ((uint64_t)b[1] << 32 | b[0]) + a - ((uint64_t)sbk[1] << 32 | sbk[0]);
    const uint64_t cc = ((uint64_t)b[3] << 32 | b[2]) + c - ((uint64_t)sbk[3] << 32 | sbk[2]);
    const uint64_t cg = ((uint64_t)b[5] << 32 | b[4]) + g - ((uint64_t)sbk[5] << 32 | sbk[4]);
    out[2 * s] = make_uint4((uint32_t)ca, (uint32_t)cc, (uint32_t)cg, 0u);
    out[2 * s + 1] = make_uint4(b[8 + 4 * h], b[9 + 4 * h], b[10 + 4 * h], b[11 + 4 * h]);
}

// Occurrence layout: 32-symbol sectors (one byte per row), or with BSB_OCC_SYM64=1 64-symbol
// sectors (half a byte per row, for an index whose 32-symbol array would not fit the device).
// Measured on GB300 the 32-symbol layout seeds faster even with the array far beyond L2: one
// sector fetch per occurrence query either way, and half the counting (100 Mb reference, 400 MB
// array: 3.08 against 3.30 ms per -K batch; 1 Gb reference, 4 GB array: 6.04 against 6.47 ms).
static int occ_layout_sym64(uint64_t seq_len)
{
    const char *e = getenv("BSB_OCC_SYM64");
    (void)seq_len;
    return e && e[0] == '1';
}

extern "C" int bsb_index_upload(bsb_ctx *ctx, const bsb_index_view_t *v)
{
    if (!ctx) return BSB_EINVAL;
    if (!v || !v->bwt || !v->sa) return bsb_fail(ctx, BSB_EINVAL, "index view is incomplete");
    if (v->sa_intv < 1 || (v->sa_intv & (v->sa_intv - 1)))
        return bsb_fail(ctx, BSB_EINVAL, "SA sample interval %d is not a power of 2", v->sa_intv);
    const uint64_t seq_len = v->L2[4];
    const uint64_t n_blocks = (seq_len + 127) / 128 + 1;
    if (v->L2[0] != 0 || v->primary > seq_len || v->bwt_size < n_blocks * 16 - 8 - 8)
        return bsb_fail(ctx, BSB_EIO, "inconsistent BWT header (seq_len %llu, %llu words)",
                        (unsigned long long)seq_len, (unsigned long long)v->bwt_size);
    if (v->n_sa != (seq_len + v->sa_intv) / v->sa_intv)
        return bsb_fail(ctx, BSB_EIO, "SA length %llu does not match seq_len", (unsigned long long)v->n_sa);
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    bsb_index_release(ctx);
    {
        // the reference blocks go to a zero-padded staging buffer of whole blocks, then are re-cut
        // into sectors (four or two per block, one extra block of padding past the last symbol)
        const size_t ref_bytes = n_blocks * 64, copy = std::min<size_t>(v->bwt_size * 4, ref_bytes);
        const int sym64 = occ_layout_sym64(seq_len);
        const uint64_t n_sectors = n_blocks * (sym64 ? 2 : 4);
        void *stage = nullptr;
        if ((rc = bsb_cuda(ctx, cudaMalloc(&ctx->idx_bwt, n_sectors * 32), "index: occurrence array"))) return rc;
        if ((rc = bsb_cuda(ctx, cudaMalloc(&stage, ref_bytes), "index: occurrence staging"))) return rc;
        rc = bsb_cuda(ctx, cudaMemsetAsync(stage, 0, ref_bytes, ctx->stream), "index memset");
        if (!rc) rc = bsb_cuda(ctx, cudaMemcpyAsync(stage, v->bwt, copy, cudaMemcpyHostToDevice, ctx->stream),
                               "index: occurrence upload");
        if (!rc && sym64) {
            // the A, C, G counts before each 2^32-row superblock: the header of its first block
            const uint64_t n_sb = (seq_len >> 32) + 1;
            std::vector<uint64_t> sb(3 * n_sb, 0);
            for (uint64_t k = 1; k < n_sb; ++k) {
                const uint64_t w = (k << 25) * 16;
                if (w + 6 > (uint64_t)v->bwt_size) break;
                for (int c = 0; c < 3; ++c) sb[3 * k + c] = (uint64_t)v->bwt[w + 2 * c + 1] << 32 | v->bwt[w + 2 * c];
            }
            rc = bsb_cuda(ctx, cudaMalloc(&ctx->idx_sb, sb.size() * 8), "index: superblock counts");
            if (!rc) rc = bsb_cuda(ctx, cudaMemcpyAsync(ctx->idx_sb, sb.data(), sb.size() * 8, cudaMemcpyHostToDevice,
                                                        ctx->stream), "index: superblock counts");
            if (!rc) rc = bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "index: superblock counts");
        }
        if (!rc) {
            if (sym64)
                occ_sectors64_kernel<<<(unsigned)((n_sectors + 255) / 256), 256, 0, ctx->stream>>>(
                    (const uint32_t *)stage, n_sectors, (uint4 *)ctx->idx_bwt);
            else
                occ_sectors_kernel<<<(unsigned)((n_sectors + 255) / 256), 256, 0, ctx->stream>>>(
                    (const uint32_t *)stage, n_sectors, (uint4 *)ctx->idx_bwt);
            rc = bsb_cuda(ctx, cudaGetLastError(), "index: occurrence sectors");
        }
        ctx->idx_sym64 = sym64;
        if (!rc) rc = bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "index: occurrence sectors");
        cudaFree(stage);
        if (rc) return rc;
    }
    if ((rc = bsb_cuda(ctx, cudaMalloc(&ctx->idx_sa, v->n_sa * 8), "index: suffix array"))) return rc;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(ctx->idx_sa, v->sa, v->n_sa * 8, cudaMemcpyHostToDevice, ctx->stream),
                       "index: SA upload")))
        return rc;
    if (v->pac && v->l_pac > 0) {
        const size_t pb = (size_t)(v->l_pac + 3) / 4;
        if ((rc = bsb_cuda(ctx, cudaMalloc(&ctx->idx_pac, pb + 64), "index: pac"))) return rc;
        if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(ctx->idx_pac, v->pac, pb, cudaMemcpyHostToDevice, ctx->stream),
                           "index: pac upload")))
            return rc;
    }
    if (v->n_seqs > 0 && v->ann_offset && v->ann_len) {
        if ((rc = bsb_cuda(ctx, cudaMalloc(&ctx->idx_ann_off, 8 * (size_t)v->n_seqs), "index: contig offsets"))) return rc;
        if ((rc = bsb_cuda(ctx, cudaMalloc(&ctx->idx_ann_len, 4 * (size_t)v->n_seqs), "index: contig lengths"))) return rc;
        if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(ctx->idx_ann_off, v->ann_offset, 8 * (size_t)v->n_seqs,
                                                cudaMemcpyHostToDevice, ctx->stream), "index: contig upload")))
            return rc;
        if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(ctx->idx_ann_len, v->ann_len, 4 * (size_t)v->n_seqs,
                                                cudaMemcpyHostToDevice, ctx->stream), "index: contig upload")))
            return rc;
        ctx->n_seqs = v->n_seqs;
    }
    ctx->primary = v->primary;
    for (int i = 0; i < 5; ++i) ctx->L2[i] = v->L2[i];
    ctx->seq_len = seq_len;
    ctx->sa_intv = v->sa_intv;
    ctx->n_sa = v->n_sa;
    ctx->l_pac = v->l_pac;
    if ((rc = bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "index upload"))) return rc;
    if ((rc = build_sa_full(ctx))) return rc;
    ctx->has_index = 1;
    return 0;
}

static bool read_all(const char *fn, std::vector<char> &buf)
{
    FILE *fp = fopen(fn, "rb");
    if (!fp) return false;
    fseek(fp, 0, SEEK_END);
    long n = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    if (n < 0) { fclose(fp); return false; }
    buf.resize((size_t)n);
    bool ok = n == 0 || fread(buf.data(), 1, (size_t)n, fp) == (size_t)n;
    fclose(fp);
    return ok;
}

extern "C" int bsb_index_load(bsb_ctx *ctx, const char *prefix)
{
    if (!ctx) return BSB_EINVAL;
    if (!prefix) return bsb_fail(ctx, BSB_EINVAL, "prefix is NULL");
    std::string p(prefix);
    std::vector<char> bw, sa, pac, ann;
    if (!read_all((p + ".bwt").c_str(), bw) || bw.size() < 40 + 4)
        return bsb_fail(ctx, BSB_EIO, "cannot read %s.bwt", prefix);
    if (!read_all((p + ".sa").c_str(), sa) || sa.size() < 56)
        return bsb_fail(ctx, BSB_EIO, "cannot read %s.sa", prefix);
    bsb_index_view_t v;
    memset(&v, 0, sizeof v);
    uint64_t h[5];
    memcpy(h, bw.data(), 40);
    v.primary = h[0];
    v.L2[0] = 0;
    for (int i = 1; i < 5; ++i) v.L2[i] = h[i];
    v.bwt = (const uint32_t *)(bw.data() + 40);
    v.bwt_size = (bw.size() - 40) / 4;
    uint64_t sh[7];
    memcpy(sh, sa.data(), 56);
    if (sh[0] != v.primary) return bsb_fail(ctx, BSB_EIO, "SA-BWT inconsistency: primary");
    if (sh[6] != v.L2[4]) return bsb_fail(ctx, BSB_EIO, "SA-BWT inconsistency: seq_len");
    v.sa_intv = (int32_t)sh[5];
    if (v.sa_intv < 1) return bsb_fail(ctx, BSB_EIO, "bad SA interval");
    v.n_sa = (v.L2[4] + v.sa_intv) / v.sa_intv;
    if ((sa.size() - 56) / 8 != v.n_sa - 1) return bsb_fail(ctx, BSB_EIO, "short .sa file");
    std::vector<uint64_t> sav(v.n_sa);
    sav[0] = (uint64_t)-1;
    memcpy(sav.data() + 1, sa.data() + 56, (v.n_sa - 1) * 8);
    v.sa = sav.data();
    std::vector<int64_t> aoff;
    std::vector<int32_t> alen;
    if (read_all((p + ".ann").c_str(), ann) && !ann.empty()) {
        // .ann (bns_dump, bntseq.c:67-84): "l_pac n_seqs seed", then per contig a
        // "gi name [anno]" line and an "offset len n_ambs" line
        ann.push_back(0);
        long long lp = 0;
        int ns = 0;
        unsigned seed = 0;
        const char *c = ann.data();
        int used = 0;
        if (sscanf(c, "%lld %d %u%n", &lp, &ns, &seed, &used) == 3 && ns > 0) {
            c += used;
            for (int i = 0; i < ns && c; ++i) {
                c = strchr(c, '\n');                      // end of the previous line
                if (!c) break;
                c = strchr(c + 1, '\n');                  // skip the name line
                if (!c) break;
                long long off = 0;
                int ln = 0, na = 0;
                if (sscanf(c + 1, "%lld %d %d%n", &off, &ln, &na, &used) != 3) break;
                aoff.push_back(off);
                alen.push_back(ln);
                c += 1 + used;
            }
            if ((int)aoff.size() != ns) return bsb_fail(ctx, BSB_EIO, "cannot parse %s.ann", prefix);
            v.n_seqs = ns;
            v.ann_offset = aoff.data();
            v.ann_len = alen.data();
        }
        if (lp > 0 && read_all((p + ".pac").c_str(), pac) && pac.size() >= (size_t)(lp + 3) / 4) {
            v.l_pac = lp;
            v.pac = (const uint8_t *)pac.data();
        }
    }
    int rc = bsb_index_upload(ctx, &v);
    if (rc) return rc;
    // the original bases, when the index has them (bwa_idx_load reads <prefix>.opac too)
    std::vector<char> opac;
    if (v.l_pac > 0 && read_all((p + ".opac").c_str(), opac) && opac.size() >= (size_t)(v.l_pac + 3) / 4)
        return bsb_index_upload_opac(ctx, (const uint8_t *)opac.data(), v.l_pac);
    return 0;
}

extern "C" int bsb_seed_batch_device(bsb_ctx *ctx, const bsb_seed_opt_t *opt, int32_t n_reads, const uint8_t *d_seqs,
                                     const int64_t *d_offs, int64_t total_bases, int32_t max_len,
                                     bsb_intv_t *d_out, int64_t *d_out_off)
{
    return bsb_seed_batch_device_m(ctx, opt, n_reads, d_seqs, d_offs, total_bases, max_len, d_out, d_out_off, 1);
}

// With mult times the per-read seed slots (seed.cu): d_out must hold seed_padded_entries(total,
// n, mult) entries.  The overflow word (bsb_seed_overflow) tells whether a read needed more.
int bsb_seed_batch_device_m(bsb_ctx *ctx, const bsb_seed_opt_t *opt, int32_t n_reads, const uint8_t *d_seqs,
                            const int64_t *d_offs, int64_t total_bases, int32_t max_len, bsb_intv_t *d_out,
                            int64_t *d_out_off, int mult)
{
    if (!ctx) return BSB_EINVAL;
    if (!ctx->has_index) return bsb_fail(ctx, BSB_ENOINDEX, "no index loaded");
    if (!opt || n_reads < 0 || max_len < 0 || total_bases < 0) return bsb_fail(ctx, BSB_EINVAL, "bad seed arguments");
    if (opt->min_seed_len < 1 || opt->split_width < 0)
        return bsb_fail(ctx, BSB_EINVAL, "bad seeding options");
    if (n_reads == 0) return 0;
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    const size_t padded = seed_padded_entries(total_bases, n_reads, mult) * sizeof(DevIntv);
    if (max_len > BSB_SEED_MAX_LEN) return bsb_fail(ctx, BSB_ETOOLONG, "max_len %d > %d", max_len, BSB_SEED_MAX_LEN);
    const DevFM F = dev_fm(ctx);
    const size_t lists = seed_scratch_bytes(seed_threads(ctx->n_sm, max_len, n_reads, F.seq_len), max_len);
    const size_t qn = seed_queue_entries(total_bases, n_reads, mult);
    const size_t tot_b = (sizeof(int) * (size_t)n_reads + 255) & ~(size_t)255;
    const size_t need = padded + lists + 256 * 6 + sizeof(int) * (2 * (size_t)n_reads + 64) + 8 * qn + tot_b +
                        sizeof(int64_t) * (size_t)scan_tmp_words(n_reads);
    if ((rc = bsb_ensure(ctx, &ctx->seed_scratch, &ctx->seed_scratch_bytes, need, "seed scratch"))) return rc;
    char *s = (char *)ctx->seed_scratch;
    void *d_padded = s;
    void *d_lists = s + ((padded + 255) & ~(size_t)255);
    int *d_count = (int *)((char *)d_lists + ((lists + 255) & ~(size_t)255));
    int *d_ctrl = d_count + ((2 * n_reads + 63) & ~63);     // two counts per read (seed_kernel's two parts)
    void *d_queue = d_ctrl + 64;                              // pass-2 work items (int2)
    int *d_tot = (int *)((char *)d_queue + ((8 * qn + 255) & ~(size_t)255));     // seeds kept per read
    int64_t *d_scan_tmp = (int64_t *)((char *)d_tot + tot_b);
    cudaError_t e = seed_launch(F, opt->min_seed_len, opt->split_factor, opt->split_width, opt->max_mem_intv, n_reads,
                                d_seqs, d_offs, max_len, d_padded, d_count, d_out_off, d_out, d_lists, d_ctrl,
                                d_queue, (int64_t)qn, d_tot, d_scan_tmp, mult, ctx->n_sm, ctx->stream);
    ctx->seed_ctrl = d_ctrl;
    return bsb_cuda(ctx, e, "seed launch");
}

extern "C" int bsb_last_seed_extensions(bsb_ctx *ctx, int64_t *n_ext)
{
    if (!ctx || !n_ext) return BSB_EINVAL;
    *n_ext = 0;
    if (!ctx->seed_ctrl) return 0;
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    uint64_t v = 0;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(&v, ctx->seed_ctrl + 4, 8, cudaMemcpyDeviceToHost, ctx->stream), "D2H ext")))
        return rc;
    if ((rc = bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "seed stats"))) return rc;
    *n_ext = (int64_t)v;
    return 0;
}

extern "C" int bsb_seed_batch(bsb_ctx *ctx, const bsb_seed_opt_t *opt, int32_t n_reads, const uint8_t *seqs,
                              const int64_t *offs, bsb_intv_t *out, int64_t max_out, int64_t *out_off)
{
    if (!ctx) return BSB_EINVAL;
    if (!ctx->has_index) return bsb_fail(ctx, BSB_ENOINDEX, "no index loaded");
    if (!opt || !offs || n_reads < 0 || (n_reads > 0 && (!seqs || !out || !out_off)))
        return bsb_fail(ctx, BSB_EINVAL, "NULL argument");
    if (n_reads == 0) {
        if (out_off) out_off[0] = 0;
        return 0;
    }
    int max_len = 0;
    for (int r = 0; r < n_reads; ++r) {
        const int64_t l = offs[r + 1] - offs[r];
        if (l < 0) return bsb_fail(ctx, BSB_EINVAL, "read %d: negative length", r);
        if (l > BSB_SEED_MAX_LEN) return bsb_fail(ctx, BSB_ETOOLONG, "read %d: length %lld > %d", r, (long long)l, BSB_SEED_MAX_LEN);
        if (l > max_len) max_len = (int)l;
    }
    const int64_t total = offs[n_reads] - offs[0];
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    const size_t off_b = sizeof(int64_t) * ((size_t)n_reads + 1);
    const size_t seq_b = ((size_t)total + 255) & ~(size_t)255;
    if ((rc = bsb_ensure(ctx, &ctx->d_in, &ctx->d_in_bytes, seq_b + 2 * off_b + 512, "seed input staging"))) return rc;
    uint8_t *d_seqs = (uint8_t *)ctx->d_in;
    int64_t *d_offs = (int64_t *)((char *)ctx->d_in + seq_b);
    int64_t *d_out_off = (int64_t *)((char *)d_offs + ((off_b + 255) & ~(size_t)255));
    // reads are uploaded relative to offs[0]
    std::vector<int64_t> rel(n_reads + 1);
    for (int r = 0; r <= n_reads; ++r) rel[r] = offs[r] - offs[0];
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(d_seqs, seqs + offs[0], total, cudaMemcpyHostToDevice, ctx->stream), "H2D reads")))
        return rc;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(d_offs, rel.data(), off_b, cudaMemcpyHostToDevice, ctx->stream), "H2D offsets")))
        return rc;
    // a read whose passes 1-2 overflow its seed slots: the batch again with twice the slots
    for (int mult = 1;; mult *= 2) {
        const size_t out_b = seed_padded_entries(total, n_reads, mult) * sizeof(bsb_intv_t);
        if ((rc = bsb_ensure(ctx, &ctx->d_out, &ctx->d_out_bytes, out_b + 256, "seed output staging"))) return rc;
        if ((rc = bsb_seed_batch_device_m(ctx, opt, n_reads, d_seqs, d_offs, total, max_len, (bsb_intv_t *)ctx->d_out,
                                          d_out_off, mult)))
            return rc;
        int ctrl[2] = {0, 0};
        if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(out_off, d_out_off, off_b, cudaMemcpyDeviceToHost, ctx->stream),
                           "D2H offsets")) ||
            (rc = bsb_cuda(ctx, cudaMemcpyAsync(ctrl, ctx->seed_ctrl, sizeof ctrl, cudaMemcpyDeviceToHost, ctx->stream),
                           "D2H ctrl")) ||
            (rc = bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "seed batch")))
            return rc;
        if (!ctrl[1]) break;
        if (mult >= kSeedSlotMultMax)
            return bsb_fail(ctx, BSB_ETOOLONG, "read %d produced more seeds than %d times its buffer holds",
                            ctrl[1] - 1, mult);
        ++ctx->seed_regrown;
    }
    if (out_off[n_reads] > max_out)
        return bsb_fail(ctx, BSB_EINVAL, "%lld seeds do not fit max_out %lld", (long long)out_off[n_reads], (long long)max_out);
    if (out_off[n_reads] > 0 &&
        (rc = bsb_cuda(ctx, cudaMemcpy(out, ctx->d_out, sizeof(bsb_intv_t) * out_off[n_reads], cudaMemcpyDeviceToHost), "D2H seeds")))
        return rc;
    return 0;
}

extern "C" int bsb_sa_batch(bsb_ctx *ctx, const uint64_t *rows, int64_t n, uint64_t *pos)
{
    if (!ctx) return BSB_EINVAL;
    if (!ctx->has_index) return bsb_fail(ctx, BSB_ENOINDEX, "no index loaded");
    if (n < 0 || (n > 0 && (!rows || !pos))) return bsb_fail(ctx, BSB_EINVAL, "bad SA arguments");
    if (n == 0) return 0;
    for (int64_t i = 0; i < n; ++i)
        if (rows[i] > ctx->seq_len) return bsb_fail(ctx, BSB_EINVAL, "row %lld beyond seq_len", (long long)i);
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    if ((rc = bsb_ensure(ctx, &ctx->d_in, &ctx->d_in_bytes, 8 * (size_t)n + 256, "SA staging"))) return rc;
    if ((rc = bsb_ensure(ctx, &ctx->d_out, &ctx->d_out_bytes, 8 * (size_t)n + 256, "SA staging"))) return rc;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(ctx->d_in, rows, 8 * n, cudaMemcpyHostToDevice, ctx->stream), "H2D rows")))
        return rc;
    if ((rc = bsb_cuda(ctx, sa_launch(dev_fm(ctx), (const uint64_t *)ctx->d_in, n, (uint64_t *)ctx->d_out, ctx->n_sm, ctx->stream),
                       "SA launch")))
        return rc;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(pos, ctx->d_out, 8 * n, cudaMemcpyDeviceToHost, ctx->stream), "D2H SA")))
        return rc;
    return bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "SA batch");
}

cudaError_t bsb_sa_launch_ctx(bsb_ctx *ctx, const uint64_t *d_rows, int64_t n, uint64_t *d_pos)
{
    return sa_launch(dev_fm(ctx), d_rows, n, d_pos, ctx->n_sm, ctx->stream);
}

extern "C" int bsb_sa_batch_device(bsb_ctx *ctx, const uint64_t *d_rows, int64_t n, uint64_t *d_pos)
{
    if (!ctx) return BSB_EINVAL;
    if (!ctx->has_index) return bsb_fail(ctx, BSB_ENOINDEX, "no index loaded");
    if (n < 0) return bsb_fail(ctx, BSB_EINVAL, "bad SA arguments");
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    return bsb_cuda(ctx, sa_launch(dev_fm(ctx), d_rows, n, d_pos, ctx->n_sm, ctx->stream), "SA launch");
}
