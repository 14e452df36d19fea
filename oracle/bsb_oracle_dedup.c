/*
 * bsb_oracle_dedup.c -- CPU oracle for the tail of mem_align1_core.
 *
 * TEST INFRASTRUCTURE ONLY.  A plain-C restatement, function by function, of
 *   mem_sort_dedup_patch   bsbolt/External/BWA/bwamem.c:441-493
 *   mem_patch_reg          bwamem.c:410-439 (its bwa_gen_cigar2 call: orc_gen_cigar2_score)
 *   ks_introsort           ksort.h:146-226, with alnreg_slt2 / alnreg_slt (bwamem.c:395-399)
 * used as the parity checker for the GPU's post-dedup regions.  Pinned by the
 * reference's own mem_sort_dedup_patch results in tests/golden/reads_*.npz
 * (arrays dedup / dedup_off).  Built with -ffp-contract=off: the reference's
 * double and float expressions are evaluated as written, without fused
 * multiply-adds.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "bsb_oracle_chain.h"
#include "bsb_oracle_cigar.h"
#include "bsb_oracle_dedup.h"

typedef int (*reg_lt_f)(const orc_reg_t *, const orc_reg_t *);

static int reg_lt_re(const orc_reg_t *a, const orc_reg_t *b) { return a->re < b->re; }   /* alnreg_slt2 */

static int reg_lt_score(const orc_reg_t *a, const orc_reg_t *b)                            /* alnreg_slt */
{
    return a->score > b->score || (a->score == b->score && (a->rb < b->rb || (a->rb == b->rb && a->qb < b->qb)));
}

static void reg_swap(orc_reg_t *a, orc_reg_t *b)
{
    orc_reg_t t = *a;
    *a = *b;
    *b = t;
}

/* __ks_insertsort (ksort.h:146-153) on [s, t) */
static void reg_insertsort(orc_reg_t *s, orc_reg_t *t, reg_lt_f lt)
{
    for (orc_reg_t *i = s + 1; i < t; ++i)
        for (orc_reg_t *j = i; j > s && lt(j, j - 1); --j) reg_swap(j, j - 1);
}

/* ks_combsort (ksort.h:154-171) */
static void reg_combsort(size_t n, orc_reg_t *a, reg_lt_f lt)
{
    const double shrink_factor = 1.2473309501039786540366528676643;
    int do_swap;
    size_t gap = n;
    do {
        if (gap > 2) {
            gap = (size_t)(gap / shrink_factor);
            if (gap == 9 || gap == 10) gap = 11;
        }
        do_swap = 0;
        for (orc_reg_t *i = a; i < a + n - gap; ++i) {
            orc_reg_t *j = i + gap;
            if (lt(j, i)) reg_swap(i, j), do_swap = 1;
        }
    } while (do_swap || gap > 2);
    if (gap != 1) reg_insertsort(a, a + n, lt);
}

/* ks_introsort (ksort.h:172-226) */
static void reg_introsort(size_t n, orc_reg_t *a, reg_lt_f lt)
{
    int d;
    struct { orc_reg_t *left, *right; int depth; } stack[64], *top = stack;
    orc_reg_t rp, *s, *t, *i, *j, *k;
    if (n < 1) return;
    if (n == 2) {
        if (lt(&a[1], &a[0])) reg_swap(&a[0], &a[1]);
        return;
    }
    for (d = 2; 1ul << d < n; ++d) {}
    s = a, t = a + (n - 1), d <<= 1;
    for (;;) {
        if (s < t) {
            if (--d == 0) {
                reg_combsort((size_t)(t - s + 1), s, lt);
                t = s;
                continue;
            }
            i = s, j = t, k = i + ((j - i) >> 1) + 1;
            if (lt(k, i)) {
                if (lt(k, j)) k = j;
            } else k = lt(j, i) ? i : j;
            rp = *k;
            if (k != t) reg_swap(k, t);
            for (;;) {
                do ++i; while (lt(i, &rp));
                do --j; while (i <= j && lt(&rp, j));
                if (j <= i) break;
                reg_swap(i, j);
            }
            reg_swap(i, t);
            if (i - s > t - i) {
                if (i - s > 16) top->left = s, top->right = i - 1, top->depth = d, ++top;
                s = t - i > 16 ? i + 1 : t;
            } else {
                if (t - i > 16) top->left = i + 1, top->right = t, top->depth = d, ++top;
                t = i - s > 16 ? i - 1 : s;
            }
        } else {
            if (top == stack) {
                reg_insertsort(a, a + n, lt);
                return;
            }
            --top, s = top->left, t = top->right, d = top->depth;
        }
    }
}

#define PATCH_MAX_R_BW 0.05f
#define PATCH_MIN_SC_RATIO 0.90f

/* mem_patch_reg (bwamem.c:410-439); the caller guarantees a->rid == b->rid, a->rb <= b->rb */
static int patch_reg(const orc_opt_t *opt, int64_t l_pac, const uint8_t *pac, const uint8_t *query,
                     const orc_reg_t *a, const orc_reg_t *b, int *_w)
{
    int w, score = 0, q_s, r_s;
    double r;
    if (a->rb < l_pac && b->rb >= l_pac) return 0;
    if (a->qb >= b->qb || a->qe >= b->qe || a->re >= b->re) return 0;
    w = (int)((a->re - b->rb) - (a->qe - b->qb));
    w = w > 0 ? w : -w;
    r = (double)(a->re - b->rb) / (b->re - a->rb) - (double)(a->qe - b->qb) / (b->qe - a->qb);
    r = r > 0. ? r : -r;
    if (a->re < b->rb || a->qe < b->qb) {
        if (w > opt->w << 1 || r >= PATCH_MAX_R_BW) return 0;
    } else if (w > opt->w << 2 || r >= PATCH_MAX_R_BW * 2) return 0;
    w += a->w + b->w;
    w = w < opt->w << 2 ? w : opt->w << 2;
    orc_gen_cigar2_score(opt->mat, opt->o_del, opt->e_del, opt->o_ins, opt->e_ins, w, l_pac, pac, b->qe - a->qb,
                         query + a->qb, a->rb, b->re, &score);
    q_s = (int)((double)(b->qe - a->qb) / ((b->qe - b->qb) + (a->qe - a->qb)) * (b->score + a->score) + .499);
    r_s = (int)((double)(b->re - a->rb) / ((b->re - b->rb) + (a->re - a->rb)) * (b->score + a->score) + .499);
    if ((double)score / (q_s > r_s ? q_s : r_s) < PATCH_MIN_SC_RATIO) return 0;
    *_w = w;
    return score;
}

int orc_sort_dedup_patch(const orc_opt_t *opt, int64_t l_pac, const uint8_t *pac, const uint8_t *query, int n,
                         orc_reg_t *a)
{
    int m, i, j;
    if (n <= 1) {                    /* bwamem.c:444: returned as they are (n_comp stays 0) */
        return n;
    }
    reg_introsort((size_t)n, a, reg_lt_re);
    for (i = 0; i < n; ++i) a[i].n_comp = 1;
    for (i = 1; i < n; ++i) {
        orc_reg_t *p = &a[i];
        if (p->rid != a[i - 1].rid || p->rb >= a[i - 1].re + opt->max_chain_gap) continue;
        for (j = i - 1; j >= 0 && p->rid == a[j].rid && p->rb < a[j].re + opt->max_chain_gap; --j) {
            orc_reg_t *q = &a[j];
            int64_t or_, oq, mr, mq;
            int score, w;
            if (q->qe == q->qb) continue;
            or_ = q->re - p->rb;
            oq = q->qb < p->qb ? q->qe - p->qb : p->qe - q->qb;
            mr = q->re - q->rb < p->re - p->rb ? q->re - q->rb : p->re - p->rb;
            mq = q->qe - q->qb < p->qe - p->qb ? q->qe - q->qb : p->qe - p->qb;
            /* float arithmetic, as the reference's float option times an int64 */
            if ((float)or_ > opt->mask_level_redun * (float)mr && (float)oq > opt->mask_level_redun * (float)mq) {
                if (p->score < q->score) {
                    p->qe = p->qb;
                    break;
                } else q->qe = q->qb;
            } else if (q->rb < p->rb && (score = patch_reg(opt, l_pac, pac, query, q, p, &w)) > 0) {
                p->n_comp += q->n_comp + 1;
                /* seedcov / sub / csub: sub and csub are zero before dedup */
                p->seedcov = p->seedcov > q->seedcov ? p->seedcov : q->seedcov;
                p->qb = q->qb, p->rb = q->rb;
                p->truesc = p->score = score;
                p->w = w;
                q->qb = q->qe;
            }
        }
    }
    for (i = 0, m = 0; i < n; ++i)
        if (a[i].qe > a[i].qb) {
            if (m != i) a[m++] = a[i];
            else ++m;
        }
    n = m;
    reg_introsort((size_t)n, a, reg_lt_score);
    for (i = 1; i < n; ++i)
        if (a[i].score == a[i - 1].score && a[i].rb == a[i - 1].rb && a[i].qb == a[i - 1].qb) a[i].qe = a[i].qb;
    for (i = 1, m = 1; i < n; ++i)
        if (a[i].qe > a[i].qb) {
            if (m != i) a[m++] = a[i];
            else ++m;
        }
    return m;
}

void orc_sort_dedup_batch(const orc_opt_t *opt, int64_t l_pac, const uint8_t *pac, int n_reads,
                          const uint8_t *seqs, const int64_t *offs, const orc_reg_t *regs_in, const int64_t *in_off,
                          orc_reg_t *regs_out, int64_t *out_off)
{
    int64_t o = 0;
    out_off[0] = 0;
    for (int r = 0; r < n_reads; ++r) {
        const int n = (int)(in_off[r + 1] - in_off[r]);
        memcpy(regs_out + o, regs_in + in_off[r], sizeof(orc_reg_t) * n);
        o += orc_sort_dedup_patch(opt, l_pac, pac, seqs + offs[r], n, regs_out + o);
        out_off[r + 1] = o;
    }
}
