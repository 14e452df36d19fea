/*
 * golden_dump.c -- records the reference's own outputs for the fixtures in
 * tests/golden/.  TEST INFRASTRUCTURE ONLY.
 *
 * Linked (oracle/Makefile.ref) against the reference objects compiled from
 * BSBolt's bsbolt/External/BWA sources, with ksw_extend2 wrapped at link
 * time (-Wl,--wrap=ksw_extend2) so the extension jobs issued inside
 * mem_chain2aln can be captured without touching the reference sources.
 *
 * Modes
 *   golden_dump ksw <in.bin> <out.bin>
 *       in:  int64 n, int64 seq_bytes, int8 mat[25], pad[7], int32 o_del,
 *            e_del, o_ins, e_ins, zdrop, pad, then n 40-byte jobs
 *            (bsb_ext_job_t), then the sequence bytes.
 *       out: n x 6 int32 from the reference ksw_extend2 (ksw.c:380-479).
 *   golden_dump reads <index prefix> <reads.bin> <out prefix> <opt.bin>
 *       reads.bin: int64 n, int64 bytes, int64 offs[n+1], then nt4 bytes of
 *       already-converted reads.  For each read: the sorted seed intervals
 *       of mem_collect_intv (taken from mem_chain's smem buffer), the chains
 *       of mem_chain + mem_chain_flt + mem_flt_chained_seeds, the pre-dedup
 *       regions of mem_chain2aln, the regions after mem_sort_dedup_patch, and
 *       every ksw_extend2 call (inputs and
 *       tuple) made while building them.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "bwa.h"
#include "bwamem.h"
#include "bwt.h"
#include "ksw.h"
#include "kvec.h"

/* defined in bwamem.c (bwamem.c:441), not declared in bwamem.h */
int mem_sort_dedup_patch(const mem_opt_t *opt, const bntseq_t *bns, const uint8_t *pac, uint8_t *query, int n,
                         mem_alnreg_t *a);

typedef struct {
    int64_t qoff, toff;
    int32_t qlen, tlen, h0, w, end_bonus, flags;
} job_t;

/* -------- ksw_extend2 capture (link-time wrap) -------------------------- */

static FILE *g_kswlog = 0;
static int32_t g_read_id = -1;

int __real_ksw_extend2(int qlen, const uint8_t *query, int tlen, const uint8_t *target, int m,
                       const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins, int w,
                       int end_bonus, int zdrop, int h0, int *qle, int *tle, int *gtle,
                       int *gscore, int *max_off);

int __wrap_ksw_extend2(int qlen, const uint8_t *query, int tlen, const uint8_t *target, int m,
                       const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins, int w,
                       int end_bonus, int zdrop, int h0, int *qle, int *tle, int *gtle,
                       int *gscore, int *max_off)
{
    int r = __real_ksw_extend2(qlen, query, tlen, target, m, mat, o_del, e_del, o_ins, e_ins, w,
                               end_bonus, zdrop, h0, qle, tle, gtle, gscore, max_off);
    if (g_kswlog) {
        int32_t hdr[10] = {g_read_id, qlen, tlen, h0, w, end_bonus, zdrop, 0, 0, 0};
        int32_t res[6] = {r, *qle, *tle, *gtle, *gscore, *max_off};
        fwrite(hdr, 4, 10, g_kswlog);
        fwrite(res, 4, 6, g_kswlog);
        fwrite(query, 1, qlen, g_kswlog);
        fwrite(target, 1, tlen, g_kswlog);
    }
    return r;
}

static void *xread(const char *fn, size_t *len)
{
    FILE *fp = fopen(fn, "rb");
    void *buf;
    if (!fp) { perror(fn); exit(2); }
    fseek(fp, 0, SEEK_END); *len = ftell(fp); fseek(fp, 0, SEEK_SET);
    buf = malloc(*len ? *len : 1);
    if (fread(buf, 1, *len, fp) != *len) { perror(fn); exit(2); }
    fclose(fp);
    return buf;
}

static int mode_ksw(const char *in, const char *outfn)
{
    size_t len;
    uint8_t *buf = (uint8_t *)xread(in, &len);
    int64_t n = ((int64_t *)buf)[0], sb = ((int64_t *)buf)[1];
    const int8_t *mat = (const int8_t *)(buf + 16);
    const int32_t *sc = (const int32_t *)(buf + 48);
    const job_t *jobs = (const job_t *)(buf + 72);
    const uint8_t *seq = buf + 72 + n * sizeof(job_t);
    int32_t *out = (int32_t *)malloc(sizeof(int32_t) * 6 * (n ? n : 1));
    int64_t i;
    FILE *fp;
    (void)sb;
    for (i = 0; i < n; ++i) {
        const job_t *j = &jobs[i];
        int32_t *o = out + 6 * i;
        o[0] = ksw_extend2(j->qlen, seq + j->qoff, j->tlen, seq + j->toff, 5, mat, sc[0], sc[1],
                           sc[2], sc[3], j->w, j->end_bonus, sc[4], j->h0,
                           &o[1], &o[2], &o[3], &o[4], &o[5]);
    }
    fp = fopen(outfn, "wb");
    fwrite(out, sizeof(int32_t) * 6, n, fp);
    fclose(fp);
    free(out); free(buf);
    return 0;
}

/* -------- per-read seeding / chaining / extension capture --------------- */

/* layout of the smem buffer mem_chain accepts as `buf` (bwamem.c:96-98) */
typedef struct { bwtintv_v mem, mem1, *tmpv[2]; } smem_buf_t;

/* mem_chain_t and mem_seed_t as declared in bwamem.c:171-185 */
typedef struct { int64_t rbeg; int32_t qbeg, len; int score; } seed_t;
typedef struct {
    int n, m, first, rid;
    uint32_t w:29, kept:2, is_alt:1;
    float frac_rep;
    int64_t pos;
    seed_t *seeds;
} chain_t;
typedef struct { size_t n, m; chain_t *a; } chain_v;

chain_v mem_chain(const mem_opt_t *opt, const bwt_t *bwt, const bntseq_t *bns, int len,
                  const uint8_t *seq, void *buf);
int mem_chain_flt(const mem_opt_t *opt, int n_chn, chain_t *a);
void mem_flt_chained_seeds(const mem_opt_t *opt, const bntseq_t *bns, const uint8_t *pac,
                           int l_query, const uint8_t *query, int n_chn, chain_t *a);
void mem_chain2aln(const mem_opt_t *opt, const bntseq_t *bns, const uint8_t *pac, int l_query,
                   const uint8_t *query, const chain_t *c, mem_alnreg_v *av);

static int mode_reads(const char *prefix, const char *readsfn, const char *outp, const char *optfn)
{
    size_t len, olen;
    uint8_t *buf = (uint8_t *)xread(readsfn, &len);
    int32_t *ov = (int32_t *)xread(optfn, &olen);
    int64_t n = ((int64_t *)buf)[0];
    const int64_t *offs = (const int64_t *)(buf + 16);
    const uint8_t *seqs = buf + 16 + 8 * (n + 1);
    bwaidx_t *idx;
    mem_opt_t *opt = mem_opt_init();
    smem_buf_t sb;
    char fn[4096];
    FILE *f_smem, *f_chain, *f_reg, *f_dedup;
    int64_t r;

    /* option overrides: a, b, o_del, e_del, o_ins, e_ins, w, zdrop, pen_clip5, pen_clip3,
     * min_seed_len, max_occ, split_width, max_mem_intv, max_chain_gap */
    opt->a = ov[0]; opt->b = ov[1]; opt->o_del = ov[2]; opt->e_del = ov[3];
    opt->o_ins = ov[4]; opt->e_ins = ov[5]; opt->w = ov[6]; opt->zdrop = ov[7];
    opt->pen_clip5 = ov[8]; opt->pen_clip3 = ov[9]; opt->min_seed_len = ov[10];
    opt->max_occ = ov[11]; opt->split_width = ov[12]; opt->max_mem_intv = ov[13];
    opt->max_chain_gap = ov[14];
    bwa_fill_scmat(opt->a, opt->b, opt->mat);

    idx = bwa_idx_load(prefix, BWA_IDX_ALL);
    if (!idx) { fprintf(stderr, "cannot load index %s\n", prefix); return 2; }
    memset(&sb, 0, sizeof(sb));
    sb.tmpv[0] = (bwtintv_v *)calloc(1, sizeof(bwtintv_v));
    sb.tmpv[1] = (bwtintv_v *)calloc(1, sizeof(bwtintv_v));

    snprintf(fn, sizeof fn, "%s.smem.bin", outp); f_smem = fopen(fn, "wb");
    snprintf(fn, sizeof fn, "%s.chain.bin", outp); f_chain = fopen(fn, "wb");
    snprintf(fn, sizeof fn, "%s.reg.bin", outp); f_reg = fopen(fn, "wb");
    snprintf(fn, sizeof fn, "%s.ksw.bin", outp); g_kswlog = fopen(fn, "wb");
    snprintf(fn, sizeof fn, "%s.dedup.bin", outp); f_dedup = fopen(fn, "wb");

    for (r = 0; r < n; ++r) {
        int l = (int)(offs[r + 1] - offs[r]), i, j;
        uint8_t *q = (uint8_t *)malloc(l + 1);
        chain_v chn;
        mem_alnreg_v regs;
        int32_t hdr[2];
        memcpy(q, seqs + offs[r], l);
        g_read_id = (int32_t)r;
        sb.mem.n = 0;
        chn = mem_chain(opt, idx->bwt, idx->bns, l, q, &sb);
        /* seeds (mem_collect_intv output, sorted); empty if l < min_seed_len */
        hdr[0] = (int32_t)r; hdr[1] = l < opt->min_seed_len ? 0 : (int32_t)sb.mem.n;
        fwrite(hdr, 4, 2, f_smem);
        if (hdr[1]) fwrite(sb.mem.a, sizeof(bwtintv_t), sb.mem.n, f_smem);
        /* chains before filtering, then after both filters */
        hdr[1] = (int32_t)chn.n;
        fwrite(hdr, 4, 2, f_chain);
        for (i = 0; i < (int)chn.n; ++i) {
            chain_t *c = &chn.a[i];
            int32_t ch[4] = {c->n, c->rid, (int32_t)c->is_alt, 0};
            fwrite(ch, 4, 4, f_chain);
            fwrite(&c->frac_rep, 4, 1, f_chain);
            fwrite(&c->pos, 8, 1, f_chain);
            fwrite(c->seeds, sizeof(seed_t), c->n, f_chain);
        }
        chn.n = mem_chain_flt(opt, (int)chn.n, chn.a);
        mem_flt_chained_seeds(opt, idx->bns, idx->pac, l, q, (int)chn.n, chn.a);
        hdr[1] = (int32_t)chn.n;
        fwrite(hdr, 4, 2, f_chain);
        for (i = 0; i < (int)chn.n; ++i) {
            chain_t *c = &chn.a[i];
            int32_t ch[4] = {c->n, c->rid, (int32_t)c->kept, (int32_t)c->w};
            fwrite(ch, 4, 4, f_chain);
            fwrite(&c->first, 4, 1, f_chain);
            fwrite(&c->pos, 8, 1, f_chain);
            fwrite(c->seeds, sizeof(seed_t), c->n, f_chain);
        }
        kv_init(regs);
        for (i = 0; i < (int)chn.n; ++i) {
            mem_chain2aln(opt, idx->bns, idx->pac, l, q, &chn.a[i], &regs);
            free(chn.a[i].seeds);
        }
        free(chn.a);
        hdr[1] = (int32_t)regs.n;
        fwrite(hdr, 4, 2, f_reg);
        for (j = 0; j < (int)regs.n; ++j) {
            mem_alnreg_t *p = &regs.a[j];
            int64_t rr[2] = {p->rb, p->re};
            int32_t v[9] = {p->qb, p->qe, p->rid, p->score, p->truesc, p->w, p->seedcov,
                            p->seedlen0, 0};
            fwrite(rr, 8, 2, f_reg);
            fwrite(v, 4, 9, f_reg);
            fwrite(&p->frac_rep, 4, 1, f_reg);
        }
        /* the reference's own mem_sort_dedup_patch on them (bwamem.c:1181), as mem_align1_core
         * calls it: the regions mem_align1_core returns */
        regs.n = mem_sort_dedup_patch(opt, idx->bns, idx->pac, q, (int)regs.n, regs.a);
        hdr[1] = (int32_t)regs.n;
        fwrite(hdr, 4, 2, f_dedup);
        for (j = 0; j < (int)regs.n; ++j) {
            mem_alnreg_t *p = &regs.a[j];
            int64_t rr[2] = {p->rb, p->re};
            int32_t v[9] = {p->qb, p->qe, p->rid, p->score, p->truesc, p->w, p->seedcov,
                            p->seedlen0, (int32_t)p->n_comp};
            fwrite(rr, 8, 2, f_dedup);
            fwrite(v, 4, 9, f_dedup);
            fwrite(&p->frac_rep, 4, 1, f_dedup);
        }
        free(regs.a);
        free(q);
    }
    fclose(f_smem); fclose(f_chain); fclose(f_reg); fclose(f_dedup); fclose(g_kswlog); g_kswlog = 0;
    bwa_idx_destroy(idx);
    free(buf); free(ov); free(opt);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc >= 4 && strcmp(argv[1], "ksw") == 0) return mode_ksw(argv[2], argv[3]);
    if (argc >= 6 && strcmp(argv[1], "reads") == 0) return mode_reads(argv[2], argv[3], argv[4], argv[5]);
    fprintf(stderr, "usage: golden_dump ksw <in> <out> | reads <idx> <reads> <outprefix> <opt>\n");
    return 1;
}
