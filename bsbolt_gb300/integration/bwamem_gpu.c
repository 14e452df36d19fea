/*
 * bwamem_gpu.c -- the BWA-side glue of the GPU path (see bwamem_gpu.h).
 *
 * Build inside the reference's BWA directory:
 *   gcc -c -O2 -I<repo>/include -I. <repo>/bsbolt_gb300/integration/bwamem_gpu.c
 * and in mem_process_seqs (bwamem.c:1336) replace
 *   kt_for(opt->n_threads, worker1, &w, (opt->flag&MEM_F_PE)? n>>1 : n);
 * with
 *   if (mem_align_batch_gpu(g_bsb, opt, bns, pac, n, seqs, w.regs) ||
 *       mem_gen_cigar_prepass_gpu(g_bsb, opt, bns, n, seqs, w.regs))
 *       err_fatal(__func__, "%s", bsb_last_error(g_bsb));
 * and link with -Wl,--wrap=bwa_gen_cigar2.
 */
#include <stdlib.h>
#include <string.h>
#include <stdint.h>

#include "bntseq.h"
#include "bwa.h"
#include "bwamem_gpu.h"

/* defined in bwamem.c (bwamem.c:441), not declared in bwamem.h */
int mem_sort_dedup_patch(const mem_opt_t *opt, const bntseq_t *bns, const uint8_t *pac, uint8_t *query, int n,
                         mem_alnreg_t *a);

void mem_opt_to_bsb(const mem_opt_t *opt, bsb_align_opt_t *o)
{
    memset(o, 0, sizeof(*o));
    o->a = opt->a; o->b = opt->b;
    o->o_del = opt->o_del; o->e_del = opt->e_del; o->o_ins = opt->o_ins; o->e_ins = opt->e_ins;
    o->w = opt->w; o->zdrop = opt->zdrop; o->pen_clip5 = opt->pen_clip5; o->pen_clip3 = opt->pen_clip3;
    o->min_seed_len = opt->min_seed_len; o->max_occ = opt->max_occ; o->max_chain_gap = opt->max_chain_gap;
    o->min_chain_weight = opt->min_chain_weight; o->max_chain_extend = opt->max_chain_extend;
    o->mask_level = opt->mask_level; o->drop_ratio = opt->drop_ratio; o->split_factor = opt->split_factor;
    o->split_width = opt->split_width; o->max_mem_intv = (int32_t)opt->max_mem_intv;
    memcpy(o->mat, opt->mat, 25);
}

int mem_align_batch_gpu(bsb_ctx *ctx, const mem_opt_t *opt, const bntseq_t *bns, const uint8_t *pac,
                        int n, bseq1_t *seqs, mem_alnreg_v *regs)
{
    bsb_align_opt_t o;
    int64_t *offs, total = 0, *roff;
    uint8_t *buf;
    bsb_reg_t *out;
    int i, j, rc;
    mem_opt_to_bsb(opt, &o);
    offs = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
    roff = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
    for (i = 0; i < n; ++i) total += seqs[i].l_seq;
    buf = (uint8_t *)malloc(total + 1);
    offs[0] = 0;
    for (i = 0; i < n; ++i) {
        char *s = seqs[i].seq;
        /* nt4 in place, as mem_align1_core does (bwamem.c:1164-1166) */
        for (j = 0; j < seqs[i].l_seq; ++j) s[j] = s[j] < 4 ? s[j] : nst_nt4_table[(int)s[j]];
        memcpy(buf + offs[i], s, seqs[i].l_seq);
        offs[i + 1] = offs[i] + seqs[i].l_seq;
    }
    /* every region comes from one extended seed, so 4 per base is a safe bound */
    out = (bsb_reg_t *)malloc(sizeof(bsb_reg_t) * (4 * total + 64 * (int64_t)n + 1));
    rc = bsb_align_regs_batch(ctx, &o, n, buf, offs, out, 4 * total + 64 * (int64_t)n, roff);
    if (rc == 0) {
        for (i = 0; i < n; ++i) {
            mem_alnreg_v *v = &regs[i];
            int k = (int)(roff[i + 1] - roff[i]);
            v->n = v->m = k;
            v->a = (mem_alnreg_t *)malloc(sizeof(mem_alnreg_t) * (k ? k : 1));
            for (j = 0; j < k; ++j) {
                const bsb_reg_t *r = &out[roff[i] + j];
                mem_alnreg_t *a = &v->a[j];
                memset(a, 0, sizeof(*a));         /* mem_chain2aln starts from zero (bwamem.c:713) */
                a->rb = r->rb; a->re = r->re; a->qb = r->qb; a->qe = r->qe;
                a->rid = r->rid; a->score = r->score; a->truesc = r->truesc; a->w = r->w;
                a->seedcov = r->seedcov; a->seedlen0 = r->seedlen0; a->frac_rep = r->frac_rep;
            }
            /* the host-side tail of mem_align1_core (bwamem.c:1181-1194) */
            v->n = mem_sort_dedup_patch(opt, bns, pac, (uint8_t *)seqs[i].seq, (int)v->n, v->a);
            for (j = 0; j < (int)v->n; ++j)
                if (v->a[j].rid >= 0 && bns->anns[v->a[j].rid].is_alt) v->a[j].is_alt = 1;
        }
    }
    free(offs); free(roff); free(buf); free(out);
    return rc;
}

/* ---- CIGAR pre-pass and the bwa_gen_cigar2 wrapper ------------------------ */

/* infer_bw (bwamem.c:796-803) */
static int glue_infer_bw(int l1, int l2, int score, int a, int q, int r)
{
    int w;
    if (l1 == l2 && l1 * a - score < (q + r - a) << 1) return 0;
    w = (int)((double)((l1 < l2 ? l1 : l2) * a - score - q) / r + 2.);
    if (w < abs(l1 - l2)) w = abs(l1 - l2);
    return w;
}

typedef struct {
    int64_t rb, re;
    int32_t l_query, w;
    const bsb_cigar_out_t *rec;
    const uint8_t *q, *oq;        /* the job's query and original-read bytes */
} cig_entry_t;

static struct {
    int64_t n, mask;
    cig_entry_t *e;
    int64_t *slot;                 /* open addressing: entry index + 1, 0 = empty */
    bsb_cigar_job_t *jobs;
    bsb_cigar_out_t *out;
    uint8_t *qbuf, *obuf, *blob;
    int8_t mat[25];
    int o_del, e_del, o_ins, e_ins;
    int64_t l_pac, crick_l;
    int64_t served;
} g_cig;

static uint64_t cig_hash(int64_t rb, int64_t re, int l, int w)
{
    uint64_t h = (uint64_t)rb * 0x9e3779b97f4a7c15ULL ^ (uint64_t)re * 0xc2b2ae3d27d4eb4fULL;
    h ^= ((uint64_t)(uint32_t)l << 32 | (uint32_t)w) * 0x165667b19e3779f9ULL;
    return h ^ (h >> 29);
}

static void cig_clear(void)
{
    free(g_cig.e); free(g_cig.slot); free(g_cig.jobs); free(g_cig.out);
    free(g_cig.qbuf); free(g_cig.obuf); free(g_cig.blob);
    memset(&g_cig, 0, sizeof g_cig);
}

void mem_gen_cigar_stats(int64_t *kept, int64_t *served)
{
    if (kept) *kept = g_cig.n;
    if (served) *served = __atomic_load_n(&g_cig.served, __ATOMIC_RELAXED);
}

int mem_gen_cigar_prepass_gpu(bsb_ctx *ctx, const mem_opt_t *opt, const bntseq_t *bns, int n, const bseq1_t *seqs,
                              const mem_alnreg_v *regs)
{
    bsb_align_opt_t o;
    int64_t n_jobs = 0, qn = 0, on = 0, cap = 0, used = 0, k, t;
    int i, j, rc;
    cig_clear();
    for (i = 0; i < n; ++i)
        for (j = 0; j < (int)regs[i].n; ++j) {
            const mem_alnreg_t *a = &regs[i].a[j];
            if (!seqs[i].oseq || a->score < opt->T || a->rb < 0 || a->qe - a->qb > BSB_CIGAR_MAX_LEN ||
                a->re - a->rb > BSB_CIGAR_MAX_LEN)
                continue;
            ++n_jobs, qn += a->qe - a->qb, on += a->qe - a->qb;
            cap += 14 * ((a->qe - a->qb) + (a->re - a->rb)) + 48;
        }
    if (n_jobs == 0) return 0;
    g_cig.jobs = (bsb_cigar_job_t *)malloc(sizeof(bsb_cigar_job_t) * n_jobs);
    g_cig.out = (bsb_cigar_out_t *)malloc(sizeof(bsb_cigar_out_t) * n_jobs);
    g_cig.qbuf = (uint8_t *)malloc(qn + 1);
    g_cig.obuf = (uint8_t *)malloc(on + 1);
    g_cig.blob = (uint8_t *)malloc(cap + 64);
    qn = on = 0;
    for (i = 0, k = 0; i < n; ++i)
        for (j = 0; j < (int)regs[i].n; ++j) {
            const mem_alnreg_t *a = &regs[i].a[j];
            bsb_cigar_job_t *jb;
            int l, w2, tmp, x;
            if (!seqs[i].oseq || a->score < opt->T || a->rb < 0 || a->qe - a->qb > BSB_CIGAR_MAX_LEN ||
                a->re - a->rb > BSB_CIGAR_MAX_LEN)
                continue;
            l = a->qe - a->qb;
            /* the band of mem_reg2aln's first bwa_gen_cigar2 call (bwamem.c:1219-1227) */
            tmp = glue_infer_bw(l, (int)(a->re - a->rb), a->truesc, opt->a, opt->o_del, opt->e_del);
            w2 = glue_infer_bw(l, (int)(a->re - a->rb), a->truesc, opt->a, opt->o_ins, opt->e_ins);
            w2 = w2 > tmp ? w2 : tmp;
            if (w2 > opt->w) w2 = w2 < a->w ? w2 : a->w;
            w2 = w2 < opt->w << 2 ? w2 : opt->w << 2;
            jb = &g_cig.jobs[k++];
            jb->rb = a->rb, jb->re = a->re, jb->l_query = l, jb->w = w2;
            /* the nt4 query from qb and the original read from its start, as mem_reg2aln
             * hands them over (bwamem.c:1211-1216, 1228) */
            jb->qoff = qn, jb->ooff = on;
            for (x = 0; x < l; ++x) {
                const int c = (uint8_t)seqs[i].seq[a->qb + x];
                g_cig.qbuf[qn++] = c < 5 ? c : nst_nt4_table[c];
            }
            for (x = 0; x < l; ++x) {
                const int c = x < seqs[i].l_seq ? (uint8_t)seqs[i].oseq[x] : 4;
                g_cig.obuf[on++] = c < 5 ? c : nst_nt4_table[c];
            }
        }
    mem_opt_to_bsb(opt, &o);
    rc = bsb_gen_cigar_batch(ctx, &o, bns->crick_l, (int32_t)n_jobs, g_cig.jobs, g_cig.qbuf, qn, g_cig.obuf, on,
                             g_cig.out, g_cig.blob, cap + 64, &used);
    if (rc) {
        cig_clear();
        return rc;
    }
    g_cig.e = (cig_entry_t *)malloc(sizeof(cig_entry_t) * n_jobs);
    for (t = 1; t < 2 * n_jobs; t <<= 1) {}
    g_cig.mask = t - 1;
    g_cig.slot = (int64_t *)calloc(t, sizeof(int64_t));
    for (k = 0; k < n_jobs; ++k) {
        const bsb_cigar_job_t *jb = &g_cig.jobs[k];
        cig_entry_t *e;
        uint64_t h;
        if (g_cig.out[k].status != BSB_CIGAR_OK) continue;
        e = &g_cig.e[g_cig.n];
        e->rb = jb->rb, e->re = jb->re, e->l_query = jb->l_query, e->w = jb->w;
        e->rec = &g_cig.out[k];
        e->q = g_cig.qbuf + jb->qoff, e->oq = g_cig.obuf + jb->ooff;
        for (h = cig_hash(e->rb, e->re, e->l_query, e->w) & g_cig.mask; g_cig.slot[h]; h = (h + 1) & g_cig.mask) {}
        g_cig.slot[h] = ++g_cig.n;
    }
    memcpy(g_cig.mat, opt->mat, 25);
    g_cig.o_del = opt->o_del, g_cig.e_del = opt->e_del, g_cig.o_ins = opt->o_ins, g_cig.e_ins = opt->e_ins;
    g_cig.l_pac = bns->l_pac, g_cig.crick_l = bns->crick_l;
    return 0;
}

uint32_t *__real_bwa_gen_cigar2(const int8_t mat[25], int o_del, int e_del, int o_ins, int e_ins, int w_, int64_t l_pac,
                                const uint8_t *pac, const uint8_t *opac, int l_query, uint8_t *query, int64_t rb,
                                int64_t re, int *score, int *n_cigar, int *NM, int64_t crick_l, uint8_t *oquery,
                                int *cg_meth, int *cg_unmeth, int *ch_meth, int *ch_unmeth);

uint32_t *__wrap_bwa_gen_cigar2(const int8_t mat[25], int o_del, int e_del, int o_ins, int e_ins, int w_, int64_t l_pac,
                                const uint8_t *pac, const uint8_t *opac, int l_query, uint8_t *query, int64_t rb,
                                int64_t re, int *score, int *n_cigar, int *NM, int64_t crick_l, uint8_t *oquery,
                                int *cg_meth, int *cg_unmeth, int *ch_meth, int *ch_unmeth)
{
    /* only the full call of mem_reg2aln (n_cigar and the methylation outputs wanted) is kept */
    if (g_cig.n && n_cigar && NM && oquery && cg_meth && cg_unmeth && ch_meth && ch_unmeth && l_query > 0 &&
        l_pac == g_cig.l_pac && crick_l == g_cig.crick_l && o_del == g_cig.o_del && e_del == g_cig.e_del &&
        o_ins == g_cig.o_ins && e_ins == g_cig.e_ins && !memcmp(mat, g_cig.mat, 25)) {
        uint64_t h;
        for (h = cig_hash(rb, re, l_query, w_) & g_cig.mask; g_cig.slot[h]; h = (h + 1) & g_cig.mask) {
            const cig_entry_t *e = &g_cig.e[g_cig.slot[h] - 1];
            if (e->rb == rb && e->re == re && e->l_query == l_query && e->w == w_ && !memcmp(e->q, query, l_query) &&
                !memcmp(e->oq, oquery, l_query)) {
                const bsb_cigar_out_t *r = e->rec;
                uint32_t *c = (uint32_t *)malloc(r->bytes);
                memcpy(c, g_cig.blob + r->off, r->bytes);
                *score = r->score, *n_cigar = r->n_cigar, *NM = r->NM;
                *cg_meth = r->cg_meth, *cg_unmeth = r->cg_unmeth, *ch_meth = r->ch_meth, *ch_unmeth = r->ch_unmeth;
                __atomic_add_fetch(&g_cig.served, 1, __ATOMIC_RELAXED);
                return c;
            }
        }
    }
    return __real_bwa_gen_cigar2(mat, o_del, e_del, o_ins, e_ins, w_, l_pac, pac, opac, l_query, query, rb, re, score,
                                 n_cigar, NM, crick_l, oquery, cg_meth, cg_unmeth, ch_meth, ch_unmeth);
}
