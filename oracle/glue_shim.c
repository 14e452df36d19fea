/*
 * glue_shim.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Lets the BWA glue (bsbolt_gb300/integration/bwamem_gpu.c) be tested on a
 * machine without a GPU: bsb_mem_align1_batch, bsb_gen_cigar_batch and
 * bsb_align2_batch are answered by the CPU oracle (whose results equal the GPU's, by the GPU tests),
 * and the worker1 call of the reference's mem_process_seqs is redirected to
 * mem_align_batch_gpu + mem_gen_cigar_prepass_gpu, and the worker2 call is
 * preceded by mem_matesw_prepass_gpu, by a link-time wrap of kt_for
 * (-Wl,--wrap=kt_for); bsb_align2_batch is answered by the oracle too;
 * bwa_gen_cigar2 and ksw_align2 are wrapped by the glue itself
 * (-Wl,--wrap=bwa_gen_cigar2, -Wl,--wrap=ksw_align2).  The reference sources stay untouched.  The
 * resulting `bwa_glue mem` must write the same SAM as the reference `bwa mem`.
 */
#include <stdlib.h>
#include <string.h>

#include "bwamem.h"
#include "bwamem_gpu.h"
#include "bsb_oracle.h"
#include "bsb_oracle_chain.h"
#include "bsb_oracle_cigar.h"
#include "bsb_oracle_sw.h"
#include "bsb_oracle_dedup.h"
#include <stdio.h>

struct bsb_ctx {
    orc_bwt_t bwt;
    orc_bns_t bns;
    orc_ann_t *anns;
    const uint8_t *opac;
    int ready;
};
static struct bsb_ctx g_ctx;

const char *bsb_last_error(const bsb_ctx *ctx) { (void)ctx; return "oracle shim failure"; }

static int shim_align(bsb_ctx *ctx, const bsb_align_opt_t *o, int32_t n_reads, const uint8_t *seqs,
                      const int64_t *offs, bsb_reg_t *regs, int64_t max_regs, int64_t *regs_off, int dedup)
{
    orc_opt_t oo;
    orc_align_out_t out;
    int rc, r;
    memset(&oo, 0, sizeof oo);
    oo.a = o->a; oo.b = o->b; oo.o_del = o->o_del; oo.e_del = o->e_del; oo.o_ins = o->o_ins; oo.e_ins = o->e_ins;
    oo.w = o->w; oo.zdrop = o->zdrop; oo.pen_clip5 = o->pen_clip5; oo.pen_clip3 = o->pen_clip3;
    oo.min_seed_len = o->min_seed_len; oo.max_occ = o->max_occ; oo.max_chain_gap = o->max_chain_gap;
    oo.min_chain_weight = o->min_chain_weight; oo.max_chain_extend = o->max_chain_extend;
    oo.mask_level = o->mask_level; oo.drop_ratio = o->drop_ratio; oo.split_factor = o->split_factor;
    oo.split_width = o->split_width; oo.max_mem_intv = o->max_mem_intv;
    oo.mask_level_redun = o->mask_level_redun;
    memcpy(oo.mat, o->mat, 25);
    rc = orc_align_regs_batch(&ctx->bwt, &ctx->bns, &oo, n_reads, seqs, offs, &out, 4);
    if (rc == 0 && dedup) {            /* mem_sort_dedup_patch per read, in place of the pre-dedup list */
        orc_reg_t *kept = (orc_reg_t *)malloc(sizeof(orc_reg_t) * (out.regs_off[n_reads] + 1));
        int64_t *kept_off = (int64_t *)malloc(sizeof(int64_t) * (n_reads + 1));
        orc_sort_dedup_batch(&oo, ctx->bns.l_pac, ctx->bns.pac, n_reads, seqs, offs, out.regs, out.regs_off, kept,
                             kept_off);
        free(out.regs);
        free(out.regs_off);
        out.regs = kept, out.regs_off = kept_off;
    }
    if (rc == 0 && out.regs_off[n_reads] > max_regs) {   /* the library's answer to a short buffer */
        for (r = 0; r <= n_reads; ++r) regs_off[r] = out.regs_off[r];
        orc_align_out_free(&out);
        return BSB_ECAPACITY;
    }
    if (rc == 0) {
        for (r = 0; r <= n_reads; ++r) regs_off[r] = out.regs_off[r];
        for (r = 0; r < out.regs_off[n_reads]; ++r) {
            const orc_reg_t *s = &out.regs[r];
            bsb_reg_t *d = &regs[r];
            memset(d, 0, sizeof(*d));
            d->rb = s->rb; d->re = s->re; d->qb = s->qb; d->qe = s->qe; d->rid = s->rid; d->score = s->score;
            d->truesc = s->truesc; d->w = s->w; d->seedcov = s->seedcov; d->seedlen0 = s->seedlen0;
            d->frac_rep = s->frac_rep; d->n_comp = s->n_comp;
        }
        /* self-check of the test: with BSB_SHIM_PERTURB set, shift the first
         * region by one base so the SAM must change if this path is live */
        if (getenv("BSB_SHIM_PERTURB") && out.regs_off[n_reads] > 0) regs[0].rb += 1, regs[0].re += 1;
    }
    orc_align_out_free(&out);
    return rc ? BSB_EINVAL : 0;
}

int bsb_align_regs_batch(bsb_ctx *ctx, const bsb_align_opt_t *o, int32_t n_reads, const uint8_t *seqs,
                         const int64_t *offs, bsb_reg_t *regs, int64_t max_regs, int64_t *regs_off)
{
    return shim_align(ctx, o, n_reads, seqs, offs, regs, max_regs, regs_off, 0);
}

int bsb_mem_align1_batch(bsb_ctx *ctx, const bsb_align_opt_t *o, int32_t n_reads, const uint8_t *seqs,
                         const int64_t *offs, bsb_reg_t *regs, int64_t max_regs, int64_t *regs_off)
{
    return shim_align(ctx, o, n_reads, seqs, offs, regs, max_regs, regs_off, 1);
}

int bsb_gen_cigar_batch(bsb_ctx *ctx, const bsb_align_opt_t *o, int64_t crick_l, int32_t n,
                        const bsb_cigar_job_t *jobs, const uint8_t *qbuf, int64_t q_bytes, const uint8_t *obuf,
                        int64_t o_bytes, bsb_cigar_out_t *out, uint8_t *blob, int64_t blob_cap, int64_t *blob_used)
{
    int64_t used, i;
    (void)q_bytes, (void)o_bytes;
    used = orc_gen_cigar_batch(o->mat, o->o_del, o->e_del, o->o_ins, o->e_ins, ctx->bns.l_pac, ctx->bns.pac, ctx->opac,
                               crick_l, n, (const orc_cigar_job_t *)jobs, qbuf, obuf, (orc_cigar_out_t *)out, blob,
                               blob_cap, 4);
    *blob_used = used;
    if (used < 0) return BSB_EINVAL;
    /* self-check of the test: with BSB_SHIM_PERTURB_CIGAR set, change one MD digit of
     * the first record that has one, so the SAM must change if records are served */
    if (getenv("BSB_SHIM_PERTURB_CIGAR"))
        for (i = 0; i < n; ++i)
            if (out[i].status == BSB_CIGAR_OK) {
                char *md = (char *)blob + out[i].off + 4 * out[i].n_cigar;
                if (md[0] >= '0' && md[0] <= '8') { md[0] += 1; break; }
            }
    return 0;
}

int bsb_align2_batch(bsb_ctx *ctx, const bsb_ext_param_t *param, const bsb_sw_job_t *jobs, int64_t n_jobs,
                     const uint8_t *seq, int64_t seq_bytes, bsb_kswr_t *out)
{
    int64_t i;
    (void)ctx, (void)seq_bytes;
    orc_align2_batch(n_jobs, (const orc_sw_job_t *)jobs, seq, param->mat, param->o_del, param->e_del, param->o_ins,
                     param->e_ins, (orc_kswr_t *)out, 4);
    /* self-check of the test: with BSB_SHIM_PERTURB_SW set, move the start of every
     * rescued hit one base right, so the SAM must change if results are served */
    if (getenv("BSB_SHIM_PERTURB_SW"))
        for (i = 0; i < n_jobs; ++i)
            if (out[i].tb >= 0 && out[i].tb < out[i].te) ++out[i].tb;
    return 0;
}

/* matesw statistics accumulated over batches (each pre-pass starts afresh) */
static int64_t g_sw_kept, g_sw_served;

static void take_sw_stats(void)
{
    int64_t kept, served;
    mem_matesw_stats(&kept, &served);
    g_sw_kept += kept, g_sw_served += served;
}

static void print_stats(void)
{
    int64_t kept, served;
    take_sw_stats();
    mem_gen_cigar_stats(&kept, &served);
    fprintf(stderr, "[bsb_glue] cigar records kept %lld served %lld passed %lld\n", (long long)kept, (long long)served,
            (long long)mem_gen_cigar_passed());
    fprintf(stderr, "[bsb_glue] matesw jobs kept %lld served %lld\n", (long long)g_sw_kept, (long long)g_sw_served);
    fprintf(stderr, "[bsb_glue] region buffer regrown %lld\n", (long long)mem_align_regrown());
}

/* worker_t of bwamem.c:1274-1285 */
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
} worker_view_t;

void __real_kt_for(int n_threads, void (*func)(void *, long, int), void *data, long n);

void __wrap_kt_for(int n_threads, void (*func)(void *, long, int), void *data, long n)
{
    static long calls = 0;
    if ((calls++ & 1) == 0) {          /* mem_process_seqs: worker1 first, then worker2 */
        worker_view_t *w = (worker_view_t *)data;
        int n_reads = (w->opt->flag & MEM_F_PE) ? (int)(n << 1) : (int)n, i;
        if (!g_ctx.ready) {
            orc_bwt_init(&g_ctx.bwt, w->bwt->primary, w->bwt->L2 + 1, w->bwt->bwt, w->bwt->bwt_size, w->bwt->sa,
                         w->bwt->n_sa, w->bwt->sa_intv);
            g_ctx.anns = (orc_ann_t *)calloc(w->bns->n_seqs, sizeof(orc_ann_t));
            for (i = 0; i < w->bns->n_seqs; ++i) {
                g_ctx.anns[i].offset = w->bns->anns[i].offset;
                g_ctx.anns[i].len = w->bns->anns[i].len;
                g_ctx.anns[i].is_alt = w->bns->anns[i].is_alt;
            }
            g_ctx.bns.l_pac = w->bns->l_pac;
            g_ctx.bns.n_seqs = w->bns->n_seqs;
            g_ctx.bns.anns = g_ctx.anns;
            g_ctx.bns.pac = w->pac;
            g_ctx.opac = w->opac;
            g_ctx.ready = 1;
            if (getenv("BSB_SHIM_STATS")) atexit(print_stats);
        }
        if (mem_align_batch_gpu(&g_ctx, w->opt, w->bns, w->pac, n_reads, w->seqs, w->regs) != 0 ||
            mem_gen_cigar_prepass_gpu(&g_ctx, w->opt, w->bns, n_reads, w->seqs, w->regs, w->n_processed) != 0)
            abort();
        return;
    }
    {                                  /* worker2: pes is set (mem_pestat or pes0) */
        worker_view_t *w = (worker_view_t *)data;
        int n_reads = (w->opt->flag & MEM_F_PE) ? (int)(n << 1) : (int)n;
        take_sw_stats();
        if (mem_matesw_prepass_gpu(&g_ctx, w->opt, w->bns, w->pac, w->pes, n_reads, w->seqs, w->regs) != 0) abort();
    }
    __real_kt_for(n_threads, func, data, n);
}

/* The input step of fastmap.c:process through the glue's FASTQ reader (bseq_fast.c), so that
 * the SAM tests run it against the stock reader's output. */
bseq1_t *__wrap_bseq_read(int64_t chunk_size, int *n_, void *ks1_, void *ks2_, int64_t *s, int conversion,
                          int undirectional, float substitution_proportion)
{
    return bseq_read_fast(chunk_size, n_, ks1_, ks2_, s, conversion, undirectional, substitution_proportion);
}

/* The output step through the glue's writer (sam_out.c) in place of samSorter, likewise. */
struct samSorter;
static char g_sam_token;

struct samSorter *__wrap_new_samSorter(bseq1_t *first_read)
{
    sam_out_begin(first_read);
    return (struct samSorter *)&g_sam_token;
}

void __wrap_samSorter_processRead(struct samSorter *ss, bseq1_t *read) { (void)ss; sam_out_read(read); }
void __wrap_samSorter_processEnd(struct samSorter *ss) { (void)ss; sam_out_end(); }
void __wrap_samSorter_delete(struct samSorter *ss) { (void)ss; }
