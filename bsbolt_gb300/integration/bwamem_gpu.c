/*
 * bwamem_gpu.c -- the BWA-side glue of the GPU path (see bwamem_gpu.h).
 *
 * Build inside the reference's BWA directory:
 *   gcc -c -O2 -I<repo>/include -I. <repo>/bsbolt_gb300/integration/bwamem_gpu.c
 * and in mem_process_seqs (bwamem.c:1336) replace
 *   kt_for(opt->n_threads, worker1, &w, (opt->flag&MEM_F_PE)? n>>1 : n);
 * with
 *   if (mem_align_batch_gpu(g_bsb, opt, bns, pac, n, seqs, w.regs))
 *       err_fatal(__func__, "%s", bsb_last_error(g_bsb));
 */
#include <stdlib.h>
#include <string.h>

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
