/*
 * bwamem_gpu_hook.c -- plugs the GPU path into an unmodified build of BSBolt's
 * BWA fork at link time, so `bwa mem` runs its worker1 pass, its CIGAR/MD/XB
 * strings and its mate-rescue Smith-Waterman on the GPU without a source edit.
 *
 * Link the BWA objects with this file, bwamem_gpu.c and libbsbgpu.so, and
 *   -Wl,--wrap=kt_for -Wl,--wrap=bwa_gen_cigar2 -Wl,--wrap=ksw_align2 -Wl,--wrap=bwa_idx_load
 * (bsbolt_gb300/integration/Makefile does this and names the result bwa_gpu).
 *
 * bwa_idx_load (bwa.c:440, called by main_mem, fastmap.c:321) is wrapped so that the CUDA
 * context starts on a second thread while the index is read from disk, and the index goes
 * to the GPU as soon as it is in memory; the thread is joined before the wrapper returns,
 * so no CUDA work is in flight when BWA goes on (or exits on an error of its own).
 *
 * kt_for is called only by mem_process_seqs (bwamem.c:1336 and :1344), twice
 * per -K batch: worker1 (mem_align1_core per read) and then, after
 * mem_pestat, worker2 (pairing, rescue, SAM).  The wrapper therefore
 *   - on the first call of a batch, runs mem_align_batch_gpu and the CIGAR
 *     pre-pass instead of worker1 (the context and the device index are made
 *     on the first batch from the arrays bwa_idx_load already holds);
 *   - on the second, runs the mate-rescue pre-pass with the batch's pes and
 *     then the reference's own worker2 loop over its threads.
 * A library error ends the run through err_fatal, as the reference ends on
 * its own errors.  BSB_GPU_DEVICE picks the CUDA device (default 0);
 * BSB_GPU_STATS=1 prints, at exit, how many CIGAR and rescue calls the GPU
 * results answered, and the time spent in the GPU passes.  bseq_read, the input
 * step of fastmap.c:process, is answered by bseq_read_fast (bseq_fast.c: the same
 * reads, parsed with a line scan and built on threads), and the samSorter calls of its
 * output step by sam_out.c (the same bytes, copied on threads, one write per batch);
 * both also take the time of those steps for the account.
 */
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include <unistd.h>

#include "bntseq.h"
#include "bwa.h"
#include "bwt.h"
#include "utils.h"
#include "bwamem_gpu.h"

/* the leading fields of worker_t (bwamem.c:1274-1285), as kt_for receives them */
typedef struct {
    const mem_opt_t *opt;
    const bwt_t *bwt;
    const bntseq_t *bns;
    const uint8_t *pac;
    const uint8_t *opac;
    const mem_pestat_t *pes;
    void **aux;
    bseq1_t *seqs;
    mem_alnreg_v *regs;
    int64_t n_processed;
} hook_worker_t;

static bsb_ctx *g_hook_ctx;
static long g_hook_calls;
static double g_t_align, g_t_cigar, g_t_sw, g_t_worker2;
static double g_t_start, g_t_load, g_t_ctx, g_t_upload;   /* index load, context, upload (wall) */
static double g_t_read, g_t_write, g_t_write0;             /* input and output steps of the pipeline */
static double g_t_first_read, g_t_last_write;              /* the pipeline's span */
static double g_t_pipe_end, g_t_idx_free, g_t_out_close;    /* after it: index freed, SAM file closed */
static double g_t_mem_end;                                  /* main_mem returned */
static double g_t_out_flush;                                /* the SAM stream flushed and synced to disk */
static long g_batches;
static int64_t g_cig_kept, g_cig_served, g_cig_passed, g_sw_kept, g_sw_served, g_reads;

static double hook_now(void)
{
    struct timeval tv;
    gettimeofday(&tv, 0);
    return tv.tv_sec + tv.tv_usec * 1e-6;
}

static void hook_take_stats(void)
{
    int64_t k, s;
    mem_gen_cigar_stats(&k, &s);
    g_cig_kept += k, g_cig_served += s, g_cig_passed += mem_gen_cigar_passed();
    mem_matesw_stats(&k, &s);
    g_sw_kept += k, g_sw_served += s;
}

static void hook_report(void)
{
    hook_take_stats();
    fprintf(stderr, "[bsb_gpu] reads %lld; GPU time: regions %.3f s, cigar %.3f s, rescue %.3f s; worker2 %.3f s\n",
            (long long)g_reads, g_t_align, g_t_cigar, g_t_sw, g_t_worker2);
    fprintf(stderr, "[bsb_gpu] cigar records kept %lld served %lld passed %lld\n", (long long)g_cig_kept,
            (long long)g_cig_served, (long long)g_cig_passed);
    fprintf(stderr, "[bsb_gpu] matesw jobs kept %lld served %lld\n", (long long)g_sw_kept, (long long)g_sw_served);
    fprintf(stderr, "[bsb_gpu] region buffer regrown %lld\n", (long long)mem_align_regrown());
    fprintf(stderr, "[bsb_gpu] start-up: index load %.3f s, GPU context %.3f s (beside the load), index upload %.3f s; "
            "%ld batches; %.3f s from the load to exit\n", g_t_load, g_t_ctx, g_t_upload, g_batches,
            g_t_start > 0 ? hook_now() - g_t_start : 0.);
    fprintf(stderr, "[bsb_gpu] host steps: reading and converting the reads %.3f s, SAM output %.3f s "
            "(each beside the other steps of the pipeline)\n", g_t_read, g_t_write);
    if (sam_out_enabled()) sam_out_report(stderr);
    if (g_t_first_read > 0.)
        fprintf(stderr, "[bsb_gpu] timeline: load to first read %.3f s, first read to last SAM output %.3f s "
                "(alignment steps %.3f s of it), last output to exit %.3f s (pipeline end %.3f s after it, "
                "index freed in %.3f s, mem command returned %.3f s after it, SAM stream flushed and synced to "
                "disk (err_fflush, utils.c:233-258) in %.3f s, closed in %.3f s)\n",
                g_t_first_read - g_t_start, g_t_last_write - g_t_first_read,
                g_t_align + g_t_cigar + g_t_sw + g_t_worker2, hook_now() - g_t_last_write,
                g_t_pipe_end > 0. ? g_t_pipe_end - g_t_last_write : 0., g_t_idx_free,
                g_t_mem_end > 0. ? g_t_mem_end - g_t_last_write : 0., g_t_out_flush, g_t_out_close);
}

/* ---- the pipeline's input and output steps (timed for the account) ---- */

static int hook_stats(void)
{
    static int on = -1;
    if (on < 0) on = getenv("BSB_GPU_STATS") != 0;
    return on;
}

/* mem's read -> align -> write pipeline (fastmap.c:352, kthread.c:119-147): each worker takes
 * one batch through the three steps and every step runs one batch at a time, in batch order
 * (ktp_worker), so the worker count changes only what overlaps.  BSB_PIPELINE_WORKERS=n sets
 * it; the default is the reference's (two; one with mem -1).  Measured on the GB300 machine, three
 * workers gained nothing (100 Mb PE: 0.61 s from the first read to the last SAM output either
 * way; RRBS: 0.69 s with two, 0.71 s with three). */
void __real_kt_pipeline(int n_threads, void *(*func)(void *, int, void *), void *shared_data, int n_steps);
void __wrap_kt_pipeline(int n_threads, void *(*func)(void *, int, void *), void *shared_data, int n_steps)
{
    const char *e = getenv("BSB_PIPELINE_WORKERS");
    int n = n_threads;
    if (e && atoi(e) >= 1) n = atoi(e) < 8 ? atoi(e) : 8;
    __real_kt_pipeline(n, func, shared_data, n_steps);
    if (hook_stats()) g_t_pipe_end = hook_now();
}

int __real_main_mem(int argc, char *argv[]);
int __wrap_main_mem(int argc, char *argv[])
{
    const int r = __real_main_mem(argc, argv);
    if (hook_stats()) g_t_mem_end = hook_now();
    return r;
}

void __real_bwa_idx_destroy(bwaidx_t *idx);
void __wrap_bwa_idx_destroy(bwaidx_t *idx)
{
    const double t0 = hook_stats() ? hook_now() : 0.;
    __real_bwa_idx_destroy(idx);
    if (t0 > 0.) g_t_idx_free += hook_now() - t0;
}

int __real_err_fflush(FILE *stream);
int __wrap_err_fflush(FILE *stream)
{
    const double t0 = hook_stats() && stream == stdout ? hook_now() : 0.;
    const int r = __real_err_fflush(stream);
    if (t0 > 0.) g_t_out_flush += hook_now() - t0;
    return r;
}

int __real_err_fclose(FILE *stream);
int __wrap_err_fclose(FILE *stream)
{
    const double t0 = hook_stats() ? hook_now() : 0.;
    const int r = __real_err_fclose(stream);
    if (t0 > 0.) g_t_out_close += hook_now() - t0;
    return r;
}


bseq1_t *__wrap_bseq_read(int64_t chunk_size, int *n_, void *ks1_, void *ks2_, int64_t *s, int conversion,
                          int undirectional, float substitution_proportion)
{
    const double t0 = hook_stats() ? hook_now() : 0.;
    if (t0 > 0. && g_t_first_read == 0.) g_t_first_read = t0;
    bseq1_t *r = bseq_read_fast(chunk_size, n_, ks1_, ks2_, s, conversion, undirectional, substitution_proportion);
    if (t0 > 0.) g_t_read += hook_now() - t0;
    return r;
}

struct samSorter;
struct samSorter *__real_new_samSorter(bseq1_t *first_read);
void __real_samSorter_processRead(struct samSorter *ss, bseq1_t *read);
void __real_samSorter_processEnd(struct samSorter *ss);
void __real_samSorter_delete(struct samSorter *ss);

/* the output step: sam_out.c in place of samSorter (BSB_SAM_WRITER=0: the reference's) */
static char g_sam_out_token;

struct samSorter *__wrap_new_samSorter(bseq1_t *first_read)
{
    if (hook_stats()) g_t_write0 = hook_now();
    if (sam_out_enabled()) {
        sam_out_begin(first_read);
        return (struct samSorter *)&g_sam_out_token;
    }
    return __real_new_samSorter(first_read);
}

void __wrap_samSorter_processRead(struct samSorter *ss, bseq1_t *read)
{
    if (ss == (struct samSorter *)&g_sam_out_token) sam_out_read(read);
    else __real_samSorter_processRead(ss, read);
}

void __wrap_samSorter_processEnd(struct samSorter *ss)
{
    if (ss == (struct samSorter *)&g_sam_out_token) sam_out_end();
    else __real_samSorter_processEnd(ss);
}

void __wrap_samSorter_delete(struct samSorter *ss)
{
    if (ss != (struct samSorter *)&g_sam_out_token) __real_samSorter_delete(ss);
    if (hook_stats() && g_t_write0 > 0.) g_t_last_write = hook_now(), g_t_write += g_t_last_write - g_t_write0;
}

static void hook_fail(bsb_ctx *ctx, int rc, const char *what)
{
    err_fatal("bwa_gpu", "%s: %s (%s)", what, ctx ? bsb_last_error(ctx) : "no context", bsb_strerror(rc));
}

static int hook_device(void)
{
    const char *dev = getenv("BSB_GPU_DEVICE");
    return dev ? atoi(dev) : 0;
}

/* The index bwa_idx_load holds (bwa.c:363-524): the occurrence array, the sampled SA, the
 * converted pac, the contig table and the original-sequence opac the methylation strings read. */
static void hook_upload(const bwt_t *bwt, const bntseq_t *bns, const uint8_t *pac, const uint8_t *opac)
{
    bsb_index_view_t v;
    int64_t *ann_off;
    int32_t *ann_len;
    int i, rc;
    ann_off = (int64_t *)malloc(sizeof(int64_t) * (bns->n_seqs + 1));
    ann_len = (int32_t *)malloc(sizeof(int32_t) * (bns->n_seqs + 1));
    for (i = 0; i < bns->n_seqs; ++i) ann_off[i] = bns->anns[i].offset, ann_len[i] = bns->anns[i].len;
    memset(&v, 0, sizeof v);
    v.primary = bwt->primary;
    for (i = 0; i < 5; ++i) v.L2[i] = bwt->L2[i];
    v.bwt = bwt->bwt, v.bwt_size = bwt->bwt_size;
    v.sa = bwt->sa, v.n_sa = bwt->n_sa, v.sa_intv = bwt->sa_intv;
    v.pac = pac, v.l_pac = bns->l_pac;
    v.n_seqs = bns->n_seqs, v.ann_offset = ann_off, v.ann_len = ann_len;
    if ((rc = bsb_index_upload(g_hook_ctx, &v))) hook_fail(g_hook_ctx, rc, "index upload");
    if (opac && (rc = bsb_index_upload_opac(g_hook_ctx, opac, bns->l_pac))) hook_fail(g_hook_ctx, rc, "opac upload");
    free(ann_off);
    free(ann_len);
    if (getenv("BSB_GPU_STATS")) atexit(hook_report);
}

static int g_boot_rc;

static void *hook_boot(void *arg)
{
    const double t0 = hook_now();
    (void)arg;
    g_boot_rc = bsb_ctx_create(hook_device(), &g_hook_ctx);
    g_t_ctx = hook_now() - t0;
    return 0;
}

bwaidx_t *__real_bwa_idx_load(const char *hint, int which);

bwaidx_t *__wrap_bwa_idx_load(const char *hint, int which)
{
    pthread_t boot;
    bwaidx_t *idx;
    const int full = (which & BWA_IDX_ALL) == BWA_IDX_ALL;   /* bwa mem's load (fastmap.c:321) */
    const double t0 = hook_now();
    int started;
    /* SAM leaves through stdout (samSorter's fputs, bs_sorter.cpp:98-124): a 16 MB buffer instead
     * of stdio's block-sized one, set before the header is printed (fastmap.c, after this load) */
    static char *sam_buf;
    if (full && !sam_buf && (sam_buf = (char *)malloc(1 << 24)) != 0) setvbuf(stdout, sam_buf, _IOFBF, 1 << 24);
    started = full && !g_hook_ctx && pthread_create(&boot, 0, hook_boot, 0) == 0;
    double t1;
    idx = __real_bwa_idx_load(hint, which);
    if (started) {
        g_t_start = t0, g_t_load = hook_now() - t0;
        pthread_join(boot, 0);
        if (g_boot_rc) hook_fail(g_hook_ctx, g_boot_rc, "GPU context");
        t1 = hook_now();
        if (idx) hook_upload(idx->bwt, idx->bns, idx->pac, idx->opac);
        g_t_upload = hook_now() - t1;
    }
    return idx;
}

/* Without the wrapped load (an index from shared memory, bwashm.c), the context and the
 * index upload happen on the first batch, from the arrays the worker sees. */
static void hook_init(const hook_worker_t *w)
{
    int rc;
    if ((rc = bsb_ctx_create(hook_device(), &g_hook_ctx))) hook_fail(g_hook_ctx, rc, "GPU context");
    hook_upload(w->bwt, w->bns, w->pac, w->opac);
}

void __real_kt_for(int n_threads, void (*func)(void *, long, int), void *data, long n);

void __wrap_kt_for(int n_threads, void (*func)(void *, long, int), void *data, long n)
{
    hook_worker_t *w = (hook_worker_t *)data;
    const int n_reads = (w->opt->flag & MEM_F_PE) ? (int)(n << 1) : (int)n;
    double t0, t1;
    int rc;
    if ((g_hook_calls++ & 1) == 0) {   /* worker1 of mem_process_seqs */
        if (!g_hook_ctx) hook_init(w);
        hook_take_stats();             /* the previous batch's counts, before the pre-passes reset them */
        t0 = hook_now();
        if ((rc = mem_align_batch_gpu(g_hook_ctx, w->opt, w->bns, w->pac, n_reads, w->seqs, w->regs)))
            hook_fail(g_hook_ctx, rc, "GPU alignment");
        t1 = hook_now();
        if ((rc = mem_gen_cigar_prepass_gpu(g_hook_ctx, w->opt, w->bns, n_reads, w->seqs, w->regs, w->n_processed)))
            hook_fail(g_hook_ctx, rc, "GPU CIGAR pre-pass");
        g_t_align += t1 - t0, g_t_cigar += hook_now() - t1, g_reads += n_reads, ++g_batches;
        return;
    }
    /* worker2: w->pes now holds mem_pestat's (or -I's) insert-size model */
    t0 = hook_now();
    if ((rc = mem_matesw_prepass_gpu(g_hook_ctx, w->opt, w->bns, w->pac, w->pes, n_reads, w->seqs, w->regs)))
        hook_fail(g_hook_ctx, rc, "GPU mate-rescue pre-pass");
    t1 = hook_now();
    g_t_sw += t1 - t0;
    __real_kt_for(n_threads, func, data, n);
    g_t_worker2 += hook_now() - t1;
}
