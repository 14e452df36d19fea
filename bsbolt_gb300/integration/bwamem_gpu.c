/*
 * bwamem_gpu.c -- the BWA-side glue of the GPU path (see bwamem_gpu.h).
 *
 * Build inside the reference's BWA directory:
 *   gcc -c -O2 -I<repo>/include -I. <repo>/bsbolt_gb300/integration/bwamem_gpu.c
 * and in mem_process_seqs (bwamem.c:1336) replace
 *   kt_for(opt->n_threads, worker1, &w, (opt->flag&MEM_F_PE)? n>>1 : n);
 * with
 *   if (mem_align_batch_gpu(g_bsb, opt, bns, pac, n, seqs, w.regs) ||
 *       mem_gen_cigar_prepass_gpu(g_bsb, opt, bns, n, seqs, w.regs, n_processed))
 *       err_fatal(__func__, "%s", bsb_last_error(g_bsb));
 * after mem_pestat (bwamem.c:1342) add
 *   if (mem_matesw_prepass_gpu(g_bsb, opt, bns, pac, pes, n, seqs, w.regs))
 *       err_fatal(__func__, "%s", bsb_last_error(g_bsb));
 * and link with -Wl,--wrap=bwa_gen_cigar2 -Wl,--wrap=ksw_align2.
 */
#include <pthread.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>

#include "bntseq.h"
#include "bwa.h"
#include "ksw.h"
#include "bwamem_gpu.h"

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
    o->mask_level_redun = opt->mask_level_redun;
    memcpy(o->mat, opt->mat, 25);
}

/* ---- the host work around each library call, on opt->n_threads threads ----
 * BWA runs this work inside worker1/worker2 on its kt_for threads; here it is split the same
 * way: items are handed out in chunks from a shared counter, and every item writes only its
 * own slots, so the result does not depend on the thread count. */
#define GLUE_MAX_THREADS 256
#define GLUE_CHUNK 512
typedef void (*glue_body_f)(void *data, int64_t i, int tid);
typedef struct {
    glue_body_f fn;
    void *data;
    int64_t n, next;
} glue_loop_t;
typedef struct {
    glue_loop_t *L;
    int tid;
} glue_worker_t;

static void *glue_worker(void *arg)
{
    const glue_worker_t *w = (const glue_worker_t *)arg;
    glue_loop_t *L = w->L;
    for (;;) {
        int64_t b = __atomic_fetch_add(&L->next, GLUE_CHUNK, __ATOMIC_RELAXED), e, i;
        if (b >= L->n) break;
        e = b + GLUE_CHUNK < L->n ? b + GLUE_CHUNK : L->n;
        for (i = b; i < e; ++i) L->fn(L->data, i, w->tid);
    }
    return 0;
}

/* fn(data, i, tid) for i in [0, n), tid < glue_threads(n_threads) */
static int glue_threads(int n_threads) { return n_threads < 1 ? 1 : n_threads > GLUE_MAX_THREADS ? GLUE_MAX_THREADS : n_threads; }

static void glue_for(int n_threads, int64_t n, glue_body_f fn, void *data)
{
    glue_loop_t L;
    glue_worker_t w[GLUE_MAX_THREADS];
    pthread_t th[GLUE_MAX_THREADS];
    int64_t chunks = (n + GLUE_CHUNK - 1) / GLUE_CHUNK;
    int t, started = 0;
    n_threads = glue_threads(n_threads);
    if (n_threads > chunks) n_threads = chunks < 1 ? 1 : (int)chunks;
    L.fn = fn, L.data = data, L.n = n, L.next = 0;
    for (t = 0; t < n_threads; ++t) w[t].L = &L, w[t].tid = t;
    for (t = 1; t < n_threads; ++t) {                  /* a thread that fails to start leaves its share to the rest */
        if (pthread_create(&th[t], 0, glue_worker, &w[t])) break;
        started = t;
    }
    glue_worker(&w[0]);
    for (t = 1; t <= started; ++t) pthread_join(th[t], 0);
}

/* Counters that worker2's threads bump on every served call: one 64-byte line per shard and a
 * shard per thread, so that no line is written by several threads or shared with the tables
 * they read (a counter next to the CIGAR table's fields made every lookup miss). */
#define GLUE_SHARDS 64
typedef struct {
    int64_t cig_served, cig_passed, sw_served;
    char pad[64 - 3 * sizeof(int64_t)];
} glue_shard_t;
static glue_shard_t g_shard[GLUE_SHARDS] __attribute__((aligned(64)));
static int g_shard_next;
static __thread int t_shard = -1;

static glue_shard_t *glue_shard(void)
{
    if (t_shard < 0) t_shard = __atomic_fetch_add(&g_shard_next, 1, __ATOMIC_RELAXED) % GLUE_SHARDS;
    return &g_shard[t_shard];
}

static int64_t glue_shard_sum(size_t field)
{
    int64_t s = 0;
    int k;
    for (k = 0; k < GLUE_SHARDS; ++k) s += __atomic_load_n((int64_t *)((char *)&g_shard[k] + field), __ATOMIC_RELAXED);
    return s;
}

static int64_t g_align_regrown;   /* batches whose region buffer had to grow */

int64_t mem_align_regrown(void) { return __atomic_load_n(&g_align_regrown, __ATOMIC_RELAXED); }

typedef struct {
    bseq1_t *seqs;
    const bntseq_t *bns;
    mem_alnreg_v *regs;
    const int64_t *offs, *roff;
    uint8_t *buf;
    const bsb_reg_t *out;
} align_batch_t;

/* nt4 in place, as mem_align1_core does (bwamem.c:1164-1166), and into the packed batch */
static void align_encode(void *data, int64_t i, int tid)
{
    align_batch_t *B = (align_batch_t *)data;
    char *s = B->seqs[i].seq;
    int j;
    (void)tid;
    for (j = 0; j < B->seqs[i].l_seq; ++j) s[j] = s[j] < 4 ? s[j] : nst_nt4_table[(int)s[j]];
    memcpy(B->buf + B->offs[i], s, B->seqs[i].l_seq);
}

/* read i's regions as mem_alnreg_t */
static void align_convert(void *data, int64_t i, int tid)
{
    align_batch_t *B = (align_batch_t *)data;
    mem_alnreg_v *v = &B->regs[i];
    const int k = (int)(B->roff[i + 1] - B->roff[i]);
    int j;
    (void)tid;
    v->n = v->m = k;
    v->a = (mem_alnreg_t *)malloc(sizeof(mem_alnreg_t) * (k ? k : 1));
    for (j = 0; j < k; ++j) {
        const bsb_reg_t *r = &B->out[B->roff[i] + j];
        mem_alnreg_t *a = &v->a[j];
        memset(a, 0, sizeof(*a));         /* mem_chain2aln starts from zero (bwamem.c:713) */
        a->rb = r->rb; a->re = r->re; a->qb = r->qb; a->qe = r->qe;
        a->rid = r->rid; a->score = r->score; a->truesc = r->truesc; a->w = r->w;
        a->seedcov = r->seedcov; a->seedlen0 = r->seedlen0; a->frac_rep = r->frac_rep;
        a->n_comp = r->n_comp;
        /* the ALT marking of mem_align1_core (bwamem.c:1189-1193) */
        if (a->rid >= 0 && B->bns->anns[a->rid].is_alt) a->is_alt = 1;
    }
}

int mem_align_batch_gpu(bsb_ctx *ctx, const mem_opt_t *opt, const bntseq_t *bns, const uint8_t *pac,
                        int n, bseq1_t *seqs, mem_alnreg_v *regs)
{
    bsb_align_opt_t o;
    align_batch_t B;
    int64_t *offs, *roff, cap;
    uint8_t *buf;
    bsb_reg_t *out;
    int i, rc;
    mem_opt_to_bsb(opt, &o);
    offs = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
    roff = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
    offs[0] = 0;
    for (i = 0; i < n; ++i) offs[i + 1] = offs[i] + seqs[i].l_seq;
    buf = (uint8_t *)malloc(offs[n] + 1);
    B.seqs = seqs, B.bns = bns, B.regs = regs, B.offs = offs, B.roff = roff, B.buf = buf, B.out = 0;
    glue_for(opt->n_threads, n, align_encode, &B);
    /* A first guess at the region count; a read in a family of many copies can have up to
     * max_occ regions per seed (bwamem.c:281-283), and then the library answers
     * BSB_ECAPACITY with the count it needs in roff[n], and the batch runs again. */
    cap = 4 * offs[n] + 64 * (int64_t)n;
    out = (bsb_reg_t *)malloc(sizeof(bsb_reg_t) * (cap + 1));
    rc = bsb_mem_align1_batch(ctx, &o, n, buf, offs, out, cap, roff);
    if (rc == BSB_ECAPACITY && roff[n] > cap) {
        __atomic_add_fetch(&g_align_regrown, 1, __ATOMIC_RELAXED);
        cap = roff[n];
        free(out);
        out = (bsb_reg_t *)malloc(sizeof(bsb_reg_t) * (cap + 1));
        rc = bsb_mem_align1_batch(ctx, &o, n, buf, offs, out, cap, roff);
    }
    if (rc == 0) {
        B.out = out;
        glue_for(opt->n_threads, n, align_convert, &B);
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
    int64_t served0, passed0;      /* the shards' totals when this batch's table was made */
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
    g_cig.served0 = glue_shard_sum(offsetof(glue_shard_t, cig_served));
    g_cig.passed0 = glue_shard_sum(offsetof(glue_shard_t, cig_passed));
}

void mem_gen_cigar_stats(int64_t *kept, int64_t *served)
{
    if (kept) *kept = g_cig.n;
    if (served) *served = glue_shard_sum(offsetof(glue_shard_t, cig_served)) - g_cig.served0;
}

int64_t mem_gen_cigar_passed(void) { return glue_shard_sum(offsetof(glue_shard_t, cig_passed)) - g_cig.passed0; }

int mem_mark_primary_se(const mem_opt_t *opt, int n, mem_alnreg_t *a, int64_t id);   /* bwamem.c:525 */

/* A region the CIGAR pre-pass prepares: its read and the fields mem_reg2aln uses. */
typedef struct {
    int64_t rb, re;
    int32_t qb, qe, truesc, w, read;
} cig_pick_t;

static int cig_eligible(const mem_opt_t *opt, const bseq1_t *s, const mem_alnreg_t *a)
{
    return s->oseq && a->score >= opt->T && a->rb >= 0 && a->qe - a->qb <= BSB_CIGAR_MAX_LEN &&
           a->re - a->rb <= BSB_CIGAR_MAX_LEN;
}

/* The regions worker2 is expected to hand to mem_reg2aln: on a copy of each read's regions,
 * mem_mark_primary_se with the id worker2 gives it (bwamem.c:1300, bwamem_pair.c:277-278),
 * then the primary and supplementary regions (mem_reg2sam, bwamem.c:1121-1128), the XA
 * candidates (mem_gen_alt's get_pri_idx and hit limits, bwamem_extra.c:91-120) and, for
 * pairs, the regions within XA_drop_ratio of the read's best when there are at most
 * CIG_PAIR_NEAR of them (mem_pair may choose any, bwamem_pair.c:188-196; in a large repeat
 * family the choice is one of hundreds and is left to the reference's function).  A region
 * that worker2 asks for and that is not here -- a mate rescue moved the marking, or the
 * pair chose another hit -- is answered by the reference's own function; with -a
 * (MEM_F_ALL) every region is prepared. */
#define CIG_PAIR_NEAR 16
typedef struct {
    const mem_opt_t *opt;
    const bseq1_t *seqs;
    const mem_alnreg_v *regs;
    int64_t n_processed;
    const int64_t *base;           /* read i's picks go to pick[base[i]..], at most regs[i].n */
    int *n_of;                     /* and their count */
    cig_pick_t *pick;
    mem_alnreg_t *tmp;             /* per-thread copies of a read's regions ... */
    int *cnt;                      /* ... and XA counts, tmax + 1 each */
    int tmax;
} cig_sel_t;

static void cig_select1(void *data, int64_t i64, int tid)
{
    cig_sel_t *S = (cig_sel_t *)data;
    const mem_opt_t *opt = S->opt;
    const int i = (int)i64, k = (int)S->regs[i].n;
    const mem_alnreg_t *a = S->regs[i].a;
    mem_alnreg_t *tmp = S->tmp + (int64_t)tid * (S->tmax + 1);
    int *cnt = S->cnt + (int64_t)tid * (S->tmax + 1);
    cig_pick_t *pick = S->pick + S->base[i];
    int near = 0, j, m = 0;
    S->n_of[i] = 0;
    if (k == 0 || !S->seqs[i].oseq) return;
    if (!(opt->flag & MEM_F_ALL)) {
        memcpy(tmp, a, sizeof(mem_alnreg_t) * k);
        mem_mark_primary_se(opt, k, tmp, S->n_processed + i);
        memset(cnt, 0, sizeof(int) * k);
        for (j = 0; j < k; ++j) {
            const int r = tmp[j].secondary_all;
            if (r >= 0 && tmp[j].score >= tmp[r].score * opt->XA_drop_ratio) ++cnt[r];
        }
        a = tmp;
        for (j = 0; j < k; ++j) near += a[j].score >= a[0].score * opt->XA_drop_ratio;
    }
    for (j = 0; j < k; ++j) {
        const mem_alnreg_t *p = &a[j];
        if (!cig_eligible(opt, &S->seqs[i], p)) continue;
        if (!(opt->flag & MEM_F_ALL) && p->secondary >= 0) {
            const int r = p->secondary_all;
            const int xa = r >= 0 && p->score >= a[r].score * opt->XA_drop_ratio && cnt[r] <= opt->max_XA_hits;
            const int pair = (opt->flag & MEM_F_PE) && near <= CIG_PAIR_NEAR &&
                             p->score >= a[0].score * opt->XA_drop_ratio;
            if (!xa && !pair) continue;
        }
        pick[m].rb = p->rb, pick[m].re = p->re, pick[m].qb = p->qb, pick[m].qe = p->qe;
        pick[m].truesc = p->truesc, pick[m].w = p->w, pick[m].read = i;
        ++m;
    }
    S->n_of[i] = m;
}

static cig_pick_t *cig_select(const mem_opt_t *opt, int n, const bseq1_t *seqs, const mem_alnreg_v *regs,
                              int64_t n_processed, int64_t *n_pick)
{
    cig_sel_t S;
    int64_t *base = (int64_t *)malloc(sizeof(int64_t) * (n + 1)), m = 0;
    int i, tmax = 0;
    base[0] = 0;
    for (i = 0; i < n; ++i) {
        base[i + 1] = base[i] + regs[i].n;
        tmax = (int)regs[i].n > tmax ? (int)regs[i].n : tmax;
    }
    S.opt = opt, S.seqs = seqs, S.regs = regs, S.n_processed = n_processed, S.base = base, S.tmax = tmax;
    S.n_of = (int *)malloc(sizeof(int) * (n + 1));
    S.pick = (cig_pick_t *)malloc(sizeof(cig_pick_t) * (base[n] + 1));
    S.tmp = (mem_alnreg_t *)malloc(sizeof(mem_alnreg_t) * (tmax + 1) * glue_threads(opt->n_threads));
    S.cnt = (int *)malloc(sizeof(int) * (tmax + 1) * glue_threads(opt->n_threads));
    glue_for(opt->n_threads, n, cig_select1, &S);
    for (i = 0; i < n; ++i) {                           /* in read order, as one pass would leave them */
        if (S.n_of[i] && m != base[i]) memmove(&S.pick[m], &S.pick[base[i]], sizeof(cig_pick_t) * S.n_of[i]);
        m += S.n_of[i];
    }
    free(S.tmp); free(S.cnt); free(S.n_of); free(base);
    *n_pick = m;
    return S.pick;
}

typedef struct {
    const mem_opt_t *opt;
    const bseq1_t *seqs;
    const cig_pick_t *pick;
} cig_pack_t;

/* job k: its band and its query bytes at the offsets set beforehand */
static void cig_pack1(void *data, int64_t k, int tid)
{
    const cig_pack_t *P = (const cig_pack_t *)data;
    const mem_opt_t *opt = P->opt;
    const cig_pick_t *a = &P->pick[k];
    const bseq1_t *s = &P->seqs[a->read];
    bsb_cigar_job_t *jb = &g_cig.jobs[k];
    uint8_t *q = g_cig.qbuf + jb->qoff, *oq = g_cig.obuf + jb->ooff;
    const int l = a->qe - a->qb;
    int w2, tmp, x;
    (void)tid;
    /* the band of mem_reg2aln's first bwa_gen_cigar2 call (bwamem.c:1219-1227) */
    tmp = glue_infer_bw(l, (int)(a->re - a->rb), a->truesc, opt->a, opt->o_del, opt->e_del);
    w2 = glue_infer_bw(l, (int)(a->re - a->rb), a->truesc, opt->a, opt->o_ins, opt->e_ins);
    w2 = w2 > tmp ? w2 : tmp;
    if (w2 > opt->w) w2 = w2 < a->w ? w2 : a->w;
    w2 = w2 < opt->w << 2 ? w2 : opt->w << 2;
    jb->rb = a->rb, jb->re = a->re, jb->l_query = l, jb->w = w2;
    /* the nt4 query from qb and the original read from its start, as mem_reg2aln
     * hands them over (bwamem.c:1211-1216, 1228) */
    for (x = 0; x < l; ++x) {
        const int c = (uint8_t)s->seq[a->qb + x];
        q[x] = c < 5 ? c : nst_nt4_table[c];
    }
    for (x = 0; x < l; ++x) {
        const int c = x < s->l_seq ? (uint8_t)s->oseq[x] : 4;
        oq[x] = c < 5 ? c : nst_nt4_table[c];
    }
}

int mem_gen_cigar_prepass_gpu(bsb_ctx *ctx, const mem_opt_t *opt, const bntseq_t *bns, int n, const bseq1_t *seqs,
                              const mem_alnreg_v *regs, int64_t n_processed)
{
    bsb_align_opt_t o;
    cig_pack_t P;
    int64_t n_jobs, qn = 0, on = 0, cap = 0, used = 0, k, t, n_pick = 0;
    int rc;
    cig_pick_t *pick;
    cig_clear();
    pick = cig_select(opt, n, seqs, regs, n_processed, &n_pick);
    n_jobs = n_pick;
    if (n_jobs == 0) {
        free(pick);
        return 0;
    }
    g_cig.jobs = (bsb_cigar_job_t *)malloc(sizeof(bsb_cigar_job_t) * n_jobs);
    for (k = 0; k < n_pick; ++k) {
        const cig_pick_t *a = &pick[k];
        g_cig.jobs[k].qoff = qn, g_cig.jobs[k].ooff = on;
        qn += a->qe - a->qb, on += a->qe - a->qb;
        cap += 14 * ((a->qe - a->qb) + (a->re - a->rb)) + 48;
    }
    g_cig.out = (bsb_cigar_out_t *)malloc(sizeof(bsb_cigar_out_t) * n_jobs);
    g_cig.qbuf = (uint8_t *)malloc(qn + 1);
    g_cig.obuf = (uint8_t *)malloc(on + 1);
    g_cig.blob = (uint8_t *)malloc(cap + 64);
    P.opt = opt, P.seqs = seqs, P.pick = pick;
    glue_for(opt->n_threads, n_pick, cig_pack1, &P);
    free(pick);
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
                __atomic_add_fetch(&glue_shard()->cig_served, 1, __ATOMIC_RELAXED);
                return c;
            }
        }
    }
    if (n_cigar && oquery) __atomic_add_fetch(&glue_shard()->cig_passed, 1, __ATOMIC_RELAXED);   /* not served */
    return __real_bwa_gen_cigar2(mat, o_del, e_del, o_ins, e_ins, w_, l_pac, pac, opac, l_query, query, rb, re, score,
                                 n_cigar, NM, crick_l, oquery, cg_meth, cg_unmeth, ch_meth, ch_unmeth);
}

/* ---- mate-rescue pre-pass and the ksw_align2 wrapper ----------------------- */

typedef struct {
    int32_t qlen, tlen, xtra, pad_;
    const uint8_t *q, *t;
    bsb_kswr_t r;
} sw_entry_t;

static struct {
    int64_t n, mask;
    sw_entry_t *e;
    int64_t *slot;                 /* open addressing: entry index + 1, 0 = empty */
    uint8_t *seq;
    int8_t mat[25];
    int o_del, e_del, o_ins, e_ins;
    int64_t served0;               /* the shards' total when this batch's table was made */
} g_sw;

/* content hash of one ksw_align2 call: lengths, flags and both sequences */
static uint64_t sw_hash(int qlen, const uint8_t *q, int tlen, const uint8_t *t, int xtra)
{
    uint64_t h = ((uint64_t)(uint32_t)qlen << 32 | (uint32_t)tlen) * 0x9e3779b97f4a7c15ULL ^ (uint32_t)xtra;
    const uint8_t *p[2] = {q, t};
    int l[2] = {qlen, tlen}, s, i;
    for (s = 0; s < 2; ++s) {
        for (i = 0; i + 8 <= l[s]; i += 8) {
            uint64_t w;
            memcpy(&w, p[s] + i, 8);
            h = (h ^ w) * 0xc2b2ae3d27d4eb4fULL;
            h ^= h >> 29;
        }
        for (; i < l[s]; ++i) h = (h ^ p[s][i]) * 0x165667b19e3779f9ULL;
    }
    return h ^ (h >> 32);
}

static void sw_clear(void)
{
    free(g_sw.e); free(g_sw.slot); free(g_sw.seq);
    memset(&g_sw, 0, sizeof g_sw);
    g_sw.served0 = glue_shard_sum(offsetof(glue_shard_t, sw_served));
}

void mem_matesw_stats(int64_t *kept, int64_t *served)
{
    if (kept) *kept = g_sw.n;
    if (served) *served = glue_shard_sum(offsetof(glue_shard_t, sw_served)) - g_sw.served0;
}

/* mem_infer_dir (bwamem_pair.c:23-30) */
static int glue_infer_dir(int64_t l_pac, int64_t b1, int64_t b2, int64_t *dist)
{
    int64_t p2;
    int r1 = (b1 >= l_pac), r2 = (b2 >= l_pac);
    p2 = r1 == r2 ? b2 : (l_pac << 1) - 1 - b2;
    *dist = p2 > b1 ? p2 - b1 : b1 - p2;
    return (r1 == r2 ? 0 : 1) ^ (p2 > b1 ? 0 : 3);
}

typedef struct {
    bsb_sw_job_t *jobs;
    int64_t n, m;
    uint8_t *seq;
    int64_t len, cap;
} sw_batch_t;

static int64_t sw_put(sw_batch_t *b, const uint8_t *s, int64_t l)
{
    int64_t off = b->len;
    if (b->len + l > b->cap) {
        b->cap = (b->len + l) * 2 + 4096;
        b->seq = (uint8_t *)realloc(b->seq, b->cap);
    }
    memcpy(b->seq + off, s, l);
    b->len += l;
    return off;
}

/* The ksw_align2 calls mem_matesw would make for the region a against the mate
 * ms whose regions are ma (bwamem_pair.c:111-154), with ma as it stands before
 * any rescue of the pair. */
static void matesw_jobs(const mem_opt_t *opt, const bntseq_t *bns, const uint8_t *pac, const mem_pestat_t pes[4],
                        const mem_alnreg_t *a, int l_ms, const uint8_t *ms, const mem_alnreg_v *ma, uint8_t *rev,
                        sw_batch_t *b)
{
    int64_t l_pac = bns->l_pac;
    int i, r, skip[4];
    for (r = 0; r < 4; ++r) skip[r] = pes[r].failed ? 1 : 0;
    for (i = 0; i < (int)ma->n; ++i) {
        int64_t dist;
        r = glue_infer_dir(l_pac, a->rb, ma->a[i].rb, &dist);
        if (dist >= pes[r].low && dist <= pes[r].high) skip[r] = 1;
    }
    if (skip[0] + skip[1] + skip[2] + skip[3] == 4) return;
    for (r = 0; r < 4; ++r) {
        int is_rev, is_larger, rid = -1;
        const uint8_t *seq;
        uint8_t *ref;
        int64_t rb, re;
        if (skip[r]) continue;
        is_rev = (r >> 1 != (r & 1));
        is_larger = !(r >> 1);
        if (is_rev) {
            for (i = 0; i < l_ms; ++i) rev[l_ms - 1 - i] = ms[i] < 4 ? 3 - ms[i] : 4;
            seq = rev;
        } else
            seq = ms;
        if (!is_rev) {
            rb = is_larger ? a->rb + pes[r].low : a->rb - pes[r].high;
            re = (is_larger ? a->rb + pes[r].high : a->rb - pes[r].low) + l_ms;
        } else {
            rb = (is_larger ? a->rb + pes[r].low : a->rb - pes[r].high) - l_ms;
            re = is_larger ? a->rb + pes[r].high : a->rb - pes[r].low;
        }
        if (rb < 0) rb = 0;
        if (re > l_pac << 1) re = l_pac << 1;
        /* rb >= re leaves the reference's rid unset: that call is left to the reference */
        if (rb >= re) continue;
        ref = bns_fetch_seq(bns, pac, &rb, (rb + re) >> 1, &re, &rid);
        if (a->rid == rid && re - rb >= opt->min_seed_len) {
            bsb_sw_job_t *j;
            if (b->n == b->m) {
                b->m = b->m ? b->m * 2 : 1024;
                b->jobs = (bsb_sw_job_t *)realloc(b->jobs, sizeof(bsb_sw_job_t) * b->m);
            }
            j = &b->jobs[b->n++];
            memset(j, 0, sizeof *j);
            j->qlen = l_ms, j->tlen = (int32_t)(re - rb);
            j->xtra = KSW_XSUBO | KSW_XSTART | (l_ms * opt->a < 250 ? KSW_XBYTE : 0) | (opt->min_seed_len * opt->a);
            j->qoff = sw_put(b, seq, l_ms);
            j->toff = sw_put(b, ref, re - rb);
        }
        free(ref);
    }
}

int mem_matesw_prepass_gpu(bsb_ctx *ctx, const mem_opt_t *opt, const bntseq_t *bns, const uint8_t *pac,
                           const mem_pestat_t pes[4], int n, const bseq1_t *seqs, const mem_alnreg_v *regs)
{
    sw_batch_t b;
    bsb_ext_param_t p;
    bsb_kswr_t *out;
    uint8_t *rev;
    int64_t k, t;
    int id, i, j, max_l = 1, rc;
    sw_clear();
    if (!(opt->flag & MEM_F_PE) || (opt->flag & MEM_F_NO_RESCUE)) return 0;
    memset(&b, 0, sizeof b);
    for (i = 0; i < n; ++i) max_l = seqs[i].l_seq > max_l ? seqs[i].l_seq : max_l;
    rev = (uint8_t *)malloc(max_l);
    /* mem_sam_pe's choice of regions to rescue from (bwamem_pair.c:265-274) */
    for (id = 0; id + 1 < n; id += 2) {
        const mem_alnreg_v *a = &regs[id];
        for (i = 0; i < 2; ++i) {
            const bseq1_t *m = &seqs[id + !i];
            int taken = 0;
            if (m->l_seq <= 0 || m->l_seq > BSB_SW_MAX_QLEN) continue;   /* left to the reference */
            for (j = 0; j < (int)a[i].n && taken < opt->max_matesw; ++j) {
                if (a[i].a[j].score < a[i].a[0].score - opt->pen_unpaired) continue;
                ++taken;
                matesw_jobs(opt, bns, pac, pes, &a[i].a[j], m->l_seq, (const uint8_t *)m->seq, &a[!i], rev, &b);
            }
        }
    }
    free(rev);
    if (b.n == 0) {
        free(b.jobs); free(b.seq);
        return 0;
    }
    memset(&p, 0, sizeof p);
    memcpy(p.mat, opt->mat, 25);
    p.o_del = opt->o_del, p.e_del = opt->e_del, p.o_ins = opt->o_ins, p.e_ins = opt->e_ins, p.zdrop = opt->zdrop;
    out = (bsb_kswr_t *)malloc(sizeof(bsb_kswr_t) * b.n);
    rc = bsb_align2_batch(ctx, &p, b.jobs, b.n, b.seq, b.len, out);
    if (rc) {
        free(b.jobs); free(b.seq); free(out);
        return rc;
    }
    g_sw.seq = b.seq;
    g_sw.e = (sw_entry_t *)malloc(sizeof(sw_entry_t) * b.n);
    for (t = 1; t < 2 * b.n; t <<= 1) {}
    g_sw.mask = t - 1;
    g_sw.slot = (int64_t *)calloc(t, sizeof(int64_t));
    for (k = 0; k < b.n; ++k) {
        const bsb_sw_job_t *jb = &b.jobs[k];
        sw_entry_t *e;
        uint64_t h;
        /* a saturated byte-lane pass is defined differently by the library: the
         * reference answers that call itself */
        if ((jb->xtra & KSW_XBYTE) && out[k].score >= 255) continue;
        e = &g_sw.e[g_sw.n];
        e->qlen = jb->qlen, e->tlen = jb->tlen, e->xtra = jb->xtra;
        e->q = g_sw.seq + jb->qoff, e->t = g_sw.seq + jb->toff;
        e->r = out[k];
        for (h = sw_hash(e->qlen, e->q, e->tlen, e->t, e->xtra) & g_sw.mask; g_sw.slot[h]; h = (h + 1) & g_sw.mask) {}
        g_sw.slot[h] = ++g_sw.n;
    }
    memcpy(g_sw.mat, opt->mat, 25);
    g_sw.o_del = opt->o_del, g_sw.e_del = opt->e_del, g_sw.o_ins = opt->o_ins, g_sw.e_ins = opt->e_ins;
    free(b.jobs); free(out);
    return 0;
}

kswr_t __real_ksw_align2(int qlen, uint8_t *query, int tlen, uint8_t *target, int m, const int8_t *mat, int o_del,
                         int e_del, int o_ins, int e_ins, int xtra, kswq_t **qry);

kswr_t __wrap_ksw_align2(int qlen, uint8_t *query, int tlen, uint8_t *target, int m, const int8_t *mat, int o_del,
                         int e_del, int o_ins, int e_ins, int xtra, kswq_t **qry)
{
    /* only a call without a query profile to keep, on the pre-pass's scoring */
    if (g_sw.n && !qry && m == 5 && o_del == g_sw.o_del && e_del == g_sw.e_del && o_ins == g_sw.o_ins &&
        e_ins == g_sw.e_ins && !memcmp(mat, g_sw.mat, 25)) {
        uint64_t h;
        for (h = sw_hash(qlen, query, tlen, target, xtra) & g_sw.mask; g_sw.slot[h]; h = (h + 1) & g_sw.mask) {
            const sw_entry_t *e = &g_sw.e[g_sw.slot[h] - 1];
            if (e->qlen == qlen && e->tlen == tlen && e->xtra == xtra && !memcmp(e->q, query, qlen) &&
                !memcmp(e->t, target, tlen)) {
                kswr_t r;
                r.score = e->r.score, r.te = e->r.te, r.qe = e->r.qe, r.score2 = e->r.score2, r.te2 = e->r.te2;
                r.tb = e->r.tb, r.qb = e->r.qb;
                __atomic_add_fetch(&glue_shard()->sw_served, 1, __ATOMIC_RELAXED);
                return r;
            }
        }
    }
    return __real_ksw_align2(qlen, query, tlen, target, m, mat, o_del, e_del, o_ins, e_ins, xtra, qry);
}
