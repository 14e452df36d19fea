/*
 * bsb_oracle_cigar.c -- CPU oracle for CIGAR / MD / XB generation.
 *
 * TEST INFRASTRUCTURE ONLY (see bsb_oracle_cigar.h).  Restates, in plain C:
 *   bns_get_seq     bsbolt/External/BWA/bntseq.c:413-434
 *   ksw_global2     bsbolt/External/BWA/ksw.c:504-606 (push_cigar :492-502)
 *   bwa_gen_cigar2  bsbolt/External/BWA/bwa.c:199-351 (getMethylationContext :180-196)
 * Where the reference reads memory it never wrote (a context window clipped
 * at a sequence end, a traceback step outside the band) the job is reported
 * with a status instead of a result: those outputs are not defined.
 */
#include "bsb_oracle_cigar.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define NEG_INF (-0x40000000)          /* MINUS_INF, ksw.c:490 */

static inline int pac_at(const uint8_t *pac, int64_t k)   /* _get_pac, bntseq.h:79 */
{
    return pac[k >> 2] >> ((~k & 3) << 1) & 3;
}

/* bns_get_seq (bntseq.c:413-434) for beg <= end: the bases of [beg, end) of the
 * doubled sequence, clamped to it; *len = 0 when the interval bridges the strands.
 * *clamped tells whether either end was clamped. */
static uint8_t *get_seq(int64_t l_pac, const uint8_t *pac, int64_t beg, int64_t end, int64_t *len, int *clamped)
{
    *clamped = 0;
    if (end > l_pac << 1) end = l_pac << 1, *clamped = 1;
    if (beg < 0) beg = 0, *clamped = 1;
    if (!(beg >= l_pac || end <= l_pac)) {
        *len = 0;
        return malloc(1);
    }
    *len = end - beg;
    uint8_t *s = malloc(end - beg > 0 ? end - beg : 1);
    if (beg >= l_pac) {                 /* reverse strand: complement of the forward bases, read backwards */
        const int64_t top = (l_pac << 1) - 1 - beg;
        for (int64_t t = 0; t < end - beg; ++t) s[t] = 3 - pac_at(pac, top - t);
    } else {
        for (int64_t t = 0; t < end - beg; ++t) s[t] = pac_at(pac, beg + t);
    }
    return s;
}

static void reverse_bytes(uint8_t *a, int64_t n)
{
    for (int64_t i = 0; i < n >> 1; ++i) {
        const uint8_t t = a[i];
        a[i] = a[n - 1 - i];
        a[n - 1 - i] = t;
    }
}

/* push_cigar (ksw.c:492-502): extend the last op or append a new one */
static void push_op(uint32_t *cigar, int *n, int op, int len)
{
    if (*n && (int)(cigar[*n - 1] & 0xf) == op) cigar[*n - 1] += (uint32_t)len << 4;
    else cigar[(*n)++] = (uint32_t)len << 4 | op;
}

int orc_ksw_global2(int qlen, const uint8_t *query, int tlen, const uint8_t *target,
                    const int8_t mat[25], int o_del, int e_del, int o_ins, int e_ins, int w,
                    int *n_cigar, uint32_t *cigar, int *band_exit)
{
    const int oe_del = o_del + e_del, oe_ins = o_ins + e_ins;
    const int n_col = qlen < 2 * w + 1 ? qlen : 2 * w + 1;
    int32_t *H = malloc(sizeof(int32_t) * (qlen + 1));   /* eh[j].h: H(i-1, j-1) at the start of cell j */
    int32_t *E = malloc(sizeof(int32_t) * (qlen + 1));   /* eh[j].e: E(i, j) */
    uint8_t *z = cigar ? malloc((size_t)n_col * (tlen > 0 ? tlen : 1)) : 0;
    if (band_exit) *band_exit = 0;
    H[0] = 0, E[0] = NEG_INF;
    for (int j = 1; j <= qlen; ++j) {
        H[j] = j <= w ? -(o_ins + e_ins * j) : NEG_INF;
        E[j] = NEG_INF;
    }
    for (int i = 0; i < tlen; ++i) {
        const int8_t *srow = mat + target[i] * 5;
        const int beg = i > w ? i - w : 0, end = i + w + 1 < qlen ? i + w + 1 : qlen;
        int32_t f = NEG_INF, hl = beg == 0 ? -(o_del + e_del * (i + 1)) : NEG_INF;
        uint8_t *zi = z ? z + (size_t)i * n_col - beg : 0;
        for (int j = beg; j < end; ++j) {
            const int32_t m = H[j] + srow[query[j]];
            int32_t e = E[j], h, t;
            int d;
            H[j] = hl;
            /* H = max(M, E, F) with M winning ties, then E over F (ksw.c:554-557) */
            if (m >= e) h = m, d = 0;
            else h = e, d = 1;
            if (h < f) h = f, d = 2;
            hl = h;
            t = m - oe_del;
            e -= e_del;
            if (e > t) d |= 1 << 2;
            else e = t;
            E[j] = e;
            t = m - oe_ins;
            f -= e_ins;
            if (f > t) d |= 2 << 4;
            else f = t;
            if (zi) zi[j] = (uint8_t)d;
        }
        H[end] = hl, E[end] = NEG_INF;
    }
    const int score = H[qlen];
    if (cigar) {
        int n = 0, which = 0, i = tlen - 1, k = (i + w + 1 < qlen ? i + w + 1 : qlen) - 1;
        int out = 0;
        while (i >= 0 && k >= 0) {
            const int beg = i > w ? i - w : 0, end = i + w + 1 < qlen ? i + w + 1 : qlen;
            if (k < beg || k >= end) { out = 1; break; }
            which = z[(size_t)i * n_col + (k - beg)] >> (which << 1) & 3;
            if (which == 0) push_op(cigar, &n, 0, 1), --i, --k;
            else if (which == 1) push_op(cigar, &n, 2, 1), --i;
            else push_op(cigar, &n, 1, 1), --k;
        }
        if (!out) {
            if (i >= 0) push_op(cigar, &n, 2, i + 1);
            if (k >= 0) push_op(cigar, &n, 1, k + 1);
            for (int a = 0; a < n >> 1; ++a) {
                const uint32_t t = cigar[a];
                cigar[a] = cigar[n - 1 - a];
                cigar[n - 1 - a] = t;
            }
        } else if (band_exit) {
            *band_exit = 1;
        }
        *n_cigar = n;
    }
    free(H), free(E), free(z);
    return score;
}

/* ---- the growable output of one job (cigar words, then the MD/XB string) ---- */

typedef struct {
    uint8_t *s;
    int64_t l, m;
} obuf_t;

static void ob_put(obuf_t *b, const void *p, int64_t n)
{
    if (b->l + n > b->m) {
        b->m = (b->l + n) * 2 + 64;
        b->s = realloc(b->s, b->m);
    }
    memcpy(b->s + b->l, p, n);
    b->l += n;
}

static void ob_char(obuf_t *b, char c) { ob_put(b, &c, 1); }

static void ob_int(obuf_t *b, int v)        /* kputw (kstring.h:62-77) for v >= 0 */
{
    char t[16];
    int n = 0;
    if (v == 0) t[n++] = '0';
    for (; v > 0; v /= 10) t[n++] = (char)('0' + v % 10);
    while (n) ob_char(b, t[--n]);
}

/* getMethylationContext (bwa.c:180-196) */
static char meth_context(int b1, int b2, int b3, int methylated, int *cg, int *ch)
{
    if (b1 == 1 && b2 == 2) return ++*cg, methylated ? 'X' : 'x';
    if (b1 == 1 && b3 == 2) return ++*ch, methylated ? 'Y' : 'y';
    return ++*ch, methylated ? 'Z' : 'z';
}

typedef struct {
    const int8_t *mat;
    int o_del, e_del, o_ins, e_ins;
    int64_t l_pac, crick_l;
    const uint8_t *pac, *opac, *qbuf, *obuf;
} gen_ctx_t;

/* bwa_gen_cigar2 (bwa.c:199-351) for one job, as mem_reg2aln calls it (bwamem.c:1228):
 * n_cigar requested, oquery the whole original read. */
static void gen_one(const gen_ctx_t *c, const orc_cigar_job_t *jb, orc_cigar_out_t *o, obuf_t *ob)
{
    const int64_t l_pac = c->l_pac, rb = jb->rb, re = jb->re;
    const int l = jb->l_query;
    memset(o, 0, sizeof *o);
    o->NM = -1;
    ob->l = 0;
    if (l <= 0 || rb >= re || (rb < l_pac && re > l_pac)) {   /* bwa.c:211 */
        o->status = ORC_CIGAR_REJECT;
        return;
    }
    const int reverse = rb > l_pac;                             /* bwa.c:212: '>' (the flips below use '>=') */
    int64_t rlen;
    int clamped;
    uint8_t *rseq = get_seq(l_pac, c->pac, rb, re, &rlen, &clamped);
    if (re - rb != rlen) {                                      /* bwa.c:215 */
        free(rseq);
        o->status = ORC_CIGAR_REJECT;
        return;
    }
    uint8_t *query = malloc(l), *oq = malloc(l);
    memcpy(query, c->qbuf + jb->qoff, l);
    memcpy(oq, c->obuf + jb->ooff, l);
    if (rb >= l_pac) reverse_bytes(query, l), reverse_bytes(rseq, rlen);
    uint32_t *cig = malloc(sizeof(uint32_t) * (l + rlen + 2));
    int n_cigar = 0, score = 0, band_exit = 0;
    if (l == re - rb && jb->w == 0) {                           /* ungapped (bwa.c:222-230) */
        cig[0] = (uint32_t)l << 4;
        n_cigar = 1;
        for (int i = 0; i < l; ++i) score += c->mat[rseq[i] * 5 + query[i]];
    } else {                                                    /* band (bwa.c:232-240) */
        const int max_ins = (int)((double)(((l + 1) >> 1) * c->mat[0] - c->o_ins) / c->e_ins + 1.);
        const int max_del = (int)((double)(((l + 1) >> 1) * c->mat[0] - c->o_del) / c->e_del + 1.);
        int max_gap = max_ins > max_del ? max_ins : max_del;
        max_gap = max_gap > 1 ? max_gap : 1;
        const int dl = abs((int)rlen - l);
        int w = (max_gap + dl + 1) >> 1;
        w = w < jb->w ? w : jb->w;
        w = w > dl + 3 ? w : dl + 3;
        score = orc_ksw_global2(l, query, (int)rlen, rseq, c->mat, c->o_del, c->e_del, c->o_ins, c->e_ins, w,
                                &n_cigar, cig, &band_exit);
    }
    o->score = score;
    o->n_cigar = n_cigar;
    if (band_exit) {
        o->status = ORC_CIGAR_BAND_EXIT;
        goto done;
    }
    ob_put(ob, cig, 4 * (int64_t)n_cigar);
    {
        const int is_crick = (rb >= c->crick_l && rb < l_pac) || rb >= c->crick_l + l_pac;   /* bwa.c:256-258 */
        const int ref_base = is_crick ? 2 : 1, methyl_base = is_crick ? 0 : 3;
        int64_t clen;
        uint8_t *cs = get_seq(l_pac, c->opac, rb - 2, re + 2, &clen, &clamped);
        if (!clen) {                                            /* bwa.c:266 */
            free(cs);
            o->status = ORC_CIGAR_NO_MD;
            goto done;
        }
        if (clamped) {
            free(cs);
            o->status = ORC_CIGAR_CLIPPED;
            ob->l = 0;
            goto done;
        }
        if (rb >= l_pac) reverse_bytes(cs, clen), reverse_bytes(oq, l);
        const char *int2base = rb < l_pac ? "ACGTN" : "TGCAN";
        obuf_t ms = {0, 0, 0};                                  /* the XB call string */
        int x = 0, y = 0, u = 0, n_mm = 0, n_gap = 0, meth_pos = 0;
        int cg_m = 0, cg_u = 0, ch_m = 0, ch_u = 0;
        for (int k = 0; k < n_cigar; ++k) {
            const int op = cig[k] & 0xf, len = cig[k] >> 4;
            if (op == 0) {
                for (int i = 0; i < len; ++i) {
                    const uint8_t *r = cs + y + i;              /* r[2] is the reference base */
                    if (r[2] == ref_base) {
                        int b1, b2, b3;
                        if (!reverse && !is_crick) b1 = r[2], b2 = r[3], b3 = r[4];
                        else if (!reverse) b1 = r[1], b2 = r[2], b3 = r[3];
                        else if (!is_crick) b1 = r[2], b2 = r[1], b3 = r[0];
                        else b1 = r[3], b2 = r[2], b3 = r[1];
                        if (oq[x + i] == ref_base || oq[x + i] == methyl_base) {
                            const int meth = oq[x + i] == ref_base;
                            const char s = meth ? meth_context(b1, b2, b3, 1, &cg_m, &ch_m)
                                                : meth_context(b1, b2, b3, 0, &cg_u, &ch_u);
                            if (meth_pos > 0) ob_int(&ms, meth_pos);
                            ob_char(&ms, s);
                            meth_pos = 0, ++u;
                        } else {
                            ob_int(ob, u);
                            ob_char(ob, int2base[r[2]]);
                            ++n_mm, ++meth_pos, u = 0;
                        }
                    } else if (oq[x + i] != r[2]) {
                        ob_int(ob, u);
                        ob_char(ob, int2base[r[2]]);
                        ++n_mm, ++meth_pos, u = 0;
                    } else {
                        ++u, ++meth_pos;
                    }
                }
                x += len, y += len;
            } else if (op == 2) {
                if (k > 0 && k < n_cigar - 1) {                 /* no MD for a leading or trailing D */
                    ob_int(ob, u);
                    ob_char(ob, '^');
                    for (int i = 0; i < len; ++i) ob_char(ob, int2base[cs[y + i + 2]]);
                    u = 0, n_gap += len;
                }
                y += len;
            } else if (op == 1) {
                x += len, n_gap += len, meth_pos += len;
            }
        }
        ob_int(ob, u);
        if (meth_pos > 0) ob_int(&ms, meth_pos);
        ob_put(ob, "\tXB:Z:", 6);
        if (ms.l) ob_put(ob, ms.s, ms.l);
        ob_char(ob, 0);
        free(ms.s);
        free(cs);
        o->NM = n_mm + n_gap;
        o->cg_meth = cg_m, o->cg_unmeth = cg_u, o->ch_meth = ch_m, o->ch_unmeth = ch_u;
        o->status = ORC_CIGAR_OK;
    }
done:
    if (o->status == ORC_CIGAR_BAND_EXIT) ob->l = 0;
    free(cig), free(query), free(oq), free(rseq);
}

typedef struct {
    const gen_ctx_t *c;
    const orc_cigar_job_t *jobs;
    orc_cigar_out_t *out;
    int64_t lo, hi;
    obuf_t all;            /* this range's bytes, jobs in order */
} range_t;

static void *run_range(void *arg)
{
    range_t *r = arg;
    obuf_t one = {0, 0, 0};
    for (int64_t i = r->lo; i < r->hi; ++i) {
        gen_one(r->c, r->jobs + i, r->out + i, &one);
        r->out[i].off = r->all.l;                /* relative to the range for now */
        r->out[i].bytes = (int32_t)one.l;
        if (one.l) ob_put(&r->all, one.s, one.l);
    }
    free(one.s);
    return 0;
}

int64_t orc_gen_cigar_batch(const int8_t mat[25], int o_del, int e_del, int o_ins, int e_ins,
                            int64_t l_pac, const uint8_t *pac, const uint8_t *opac, int64_t crick_l,
                            int64_t n, const orc_cigar_job_t *jobs, const uint8_t *qbuf,
                            const uint8_t *obuf, orc_cigar_out_t *out, uint8_t *blob,
                            int64_t blob_cap, int n_threads)
{
    gen_ctx_t c = {mat, o_del, e_del, o_ins, e_ins, l_pac, crick_l, pac, opac, qbuf, obuf};
    if (n_threads < 1) n_threads = 1;
    if (n_threads > n) n_threads = n > 0 ? (int)n : 1;
    range_t *rs = calloc(n_threads, sizeof(range_t));
    pthread_t *th = calloc(n_threads, sizeof(pthread_t));
    for (int t = 0; t < n_threads; ++t) {
        rs[t].c = &c, rs[t].jobs = jobs, rs[t].out = out;
        rs[t].lo = n * t / n_threads, rs[t].hi = n * (t + 1) / n_threads;
    }
    for (int t = 1; t < n_threads; ++t) pthread_create(&th[t], 0, run_range, &rs[t]);
    run_range(&rs[0]);
    for (int t = 1; t < n_threads; ++t) pthread_join(th[t], 0);
    int64_t used = 0;
    for (int t = 0; t < n_threads; ++t) used += rs[t].all.l;
    if (used <= blob_cap) {
        int64_t base = 0;
        for (int t = 0; t < n_threads; ++t) {
            for (int64_t i = rs[t].lo; i < rs[t].hi; ++i) out[i].off += base;
            if (rs[t].all.l) memcpy(blob + base, rs[t].all.s, rs[t].all.l);
            base += rs[t].all.l;
        }
    }
    for (int t = 0; t < n_threads; ++t) free(rs[t].all.s);
    free(rs), free(th);
    return used <= blob_cap ? used : -1;
}

/* bwa_gen_cigar2 (bwa.c:199-244, 343-346) as mem_patch_reg calls it (bwamem.c:432): only
 * the score is wanted (n_cigar, NM, oquery NULL).  Returns 0 where the reference returns
 * before setting *score (bwa.c:211, 215), else 1. */
int orc_gen_cigar2_score(const int8_t mat[25], int o_del, int e_del, int o_ins, int e_ins, int w_, int64_t l_pac,
                         const uint8_t *pac, int l_query, const uint8_t *query_in, int64_t rb, int64_t re, int *score)
{
    if (l_query <= 0 || rb >= re || (rb < l_pac && re > l_pac)) return 0;
    int64_t rlen;
    int clamped;
    uint8_t *rseq = get_seq(l_pac, pac, rb, re, &rlen, &clamped);
    if (re - rb != rlen) {
        free(rseq);
        return 0;
    }
    uint8_t *query = malloc(l_query);
    memcpy(query, query_in, l_query);
    if (rb >= l_pac) reverse_bytes(query, l_query), reverse_bytes(rseq, rlen);
    if (l_query == re - rb && w_ == 0) {
        *score = 0;
        for (int i = 0; i < l_query; ++i) *score += mat[rseq[i] * 5 + query[i]];
    } else {
        const int max_ins = (int)((double)(((l_query + 1) >> 1) * mat[0] - o_ins) / e_ins + 1.);
        const int max_del = (int)((double)(((l_query + 1) >> 1) * mat[0] - o_del) / e_del + 1.);
        int max_gap = max_ins > max_del ? max_ins : max_del;
        max_gap = max_gap > 1 ? max_gap : 1;
        const int dl = abs((int)rlen - l_query);
        int w = (max_gap + dl + 1) >> 1;
        w = w < w_ ? w : w_;
        w = w > dl + 3 ? w : dl + 3;
        *score = orc_ksw_global2(l_query, query, (int)rlen, rseq, mat, o_del, e_del, o_ins, e_ins, w, 0, 0, 0);
    }
    free(query);
    free(rseq);
    return 1;
}
