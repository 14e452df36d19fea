/*
 * bsb_oracle.c -- CPU oracle (test infrastructure only; see bsb_oracle.h).
 *
 * A restatement, in our own code, of the reference algorithms on the
 * bisulfite seed/extend path of BSBolt's BWA fork (bsbolt/External/BWA).
 * It exists to check the CUDA path and to time a CPU baseline; the product
 * library never links it.  It is pinned against the reference compiled from
 * its own sources (oracle/Makefile.ref) by the fixtures in tests/golden/.
 */
#include "bsb_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ======================================================================== */
/* ksw_extend2 -- bsbolt/External/BWA/ksw.c:380-479                         */
/* ======================================================================== */

/*
 * Row-major banded DP.  H, E live in two arrays indexed by query column as in
 * the reference's eh_t array (ksw.c:376-378): before row i, Hc[j] holds
 * H(i-1, j-1) and Ec[j] holds E(i, j).  Entries outside the current band
 * keep whatever an earlier row wrote there; the band can grow back over
 * them (ksw.c:466-469), so the stale values are part of the semantics.
 */
int orc_ksw_extend2(int qlen, const uint8_t *query, int tlen, const uint8_t *target,
                    const int8_t mat[25], int o_del, int e_del, int o_ins, int e_ins,
                    int w, int end_bonus, int zdrop, int h0,
                    int *qle_, int *tle_, int *gtle_, int *gscore_, int *max_off_,
                    int64_t *cells_)
{
    const int oe_del = o_del + e_del, oe_ins = o_ins + e_ins;
    int32_t *Hc = (int32_t *)calloc((size_t)qlen + 1, sizeof(int32_t));
    int32_t *Ec = (int32_t *)calloc((size_t)qlen + 1, sizeof(int32_t));
    int8_t *prof = (int8_t *)malloc((size_t)qlen * 5 + 1);
    int64_t cells = 0;
    int i, j, c, best, best_i = -1, best_j = -1, max_ie = -1, gscore = -1, max_off = 0;
    int beg = 0, end = qlen, mat_max = 0;

    /* query profile: prof[c*qlen + j] = score of target base c vs query[j] (ksw.c:390-393) */
    for (c = 0; c < 5; ++c)
        for (j = 0; j < qlen; ++j) prof[c * qlen + j] = mat[c * 5 + query[j]];

    /* first row from h0 with an insertion run (ksw.c:395-397) */
    Hc[0] = h0;
    if (qlen >= 1) Hc[1] = h0 > oe_ins ? h0 - oe_ins : 0;
    for (j = 2; j <= qlen && Hc[j - 1] > e_ins; ++j) Hc[j] = Hc[j - 1] - e_ins;

    /* clamp the band by the longest gap that can still pay off (ksw.c:399-407);
     * the double arithmetic and the truncating casts are kept as they are */
    for (i = 0; i < 25; ++i) mat_max = mat_max > mat[i] ? mat_max : mat[i];
    {
        int max_ins = (int)((double)(qlen * mat_max + end_bonus - o_ins) / e_ins + 1.);
        int max_del = (int)((double)(qlen * mat_max + end_bonus - o_del) / e_del + 1.);
        if (max_ins < 1) max_ins = 1;
        if (max_del < 1) max_del = 1;
        if (w > max_ins) w = max_ins;
        if (w > max_del) w = max_del;
    }

    best = h0;
    for (i = 0; i < tlen; ++i) {
        const int8_t *q = &prof[target[i] * qlen];
        int f = 0, h_prev, row_max = 0, row_j = -1, jl;
        /* band for this row (ksw.c:417-419) */
        if (beg < i - w) beg = i - w;
        if (end > i + w + 1) end = i + w + 1;
        if (end > qlen) end = qlen;
        /* column -1 of this row (ksw.c:421-424) */
        if (beg == 0) {
            h_prev = h0 - (o_del + e_del * (i + 1));
            if (h_prev < 0) h_prev = 0;
        } else h_prev = 0;
        for (j = beg; j < end; ++j) {
            /* Hc[j] = H(i-1,j-1), Ec[j] = E(i,j), f = F(i,j), h_prev = H(i,j-1) (ksw.c:425-447) */
            int M = Hc[j], e = Ec[j], h, t;
            Hc[j] = h_prev;
            M = M ? M + q[j] : 0;
            h = M > e ? M : e;
            h = h > f ? h : f;
            h_prev = h;
            if (h >= row_max) row_j = j;   /* ties move to the later column */
            if (h > row_max) row_max = h;
            t = M - oe_del; if (t < 0) t = 0;
            e -= e_del; if (e < t) e = t;
            Ec[j] = e;
            t = M - oe_ins; if (t < 0) t = 0;
            f -= e_ins; if (f < t) f = t;
        }
        if (end > beg) cells += end - beg;
        jl = beg < end ? end : beg;   /* value of j after the reference's loop */
        Hc[end] = h_prev; Ec[end] = 0;
        if (jl == qlen) {             /* reached the query end (ksw.c:450-453) */
            if (!(gscore > h_prev)) max_ie = i;
            if (gscore < h_prev) gscore = h_prev;
        }
        if (row_max == 0) break;      /* ksw.c:454 */
        if (row_max > best) {
            int d = row_j - i; if (d < 0) d = -d;
            best = row_max, best_i = i, best_j = row_j;
            if (max_off < d) max_off = d;
        } else if (zdrop > 0) {        /* z-drop (ksw.c:458-464) */
            int di = i - best_i, dj = row_j - best_j;
            if (di > dj) {
                if (best - row_max - (di - dj) * e_del > zdrop) break;
            } else {
                if (best - row_max - (dj - di) * e_ins > zdrop) break;
            }
        }
        /* shrink the band to non-zero cells (ksw.c:466-469) */
        for (j = beg; j < end && Hc[j] == 0 && Ec[j] == 0; ++j) ;
        beg = j;
        for (j = end; j >= beg && Hc[j] == 0 && Ec[j] == 0; --j) ;
        end = j + 2 < qlen ? j + 2 : qlen;
    }
    free(Hc); free(Ec); free(prof);
    if (qle_) *qle_ = best_j + 1;
    if (tle_) *tle_ = best_i + 1;
    if (gtle_) *gtle_ = max_ie + 1;
    if (gscore_) *gscore_ = gscore;
    if (max_off_) *max_off_ = max_off;
    if (cells_) *cells_ = cells;
    return best;
}

typedef struct {
    int64_t qoff, toff;
    int32_t qlen, tlen, h0, w, end_bonus, pad;
} orc_job_t;

typedef struct {
    int64_t lo, hi;
    const orc_job_t *jobs;
    const uint8_t *seq;
    const int8_t *mat;
    int o_del, e_del, o_ins, e_ins, zdrop;
    int32_t *out;
    int64_t *cells;
    int64_t total;
} ksw_slice_t;

static void *ksw_slice_run(void *arg)
{
    ksw_slice_t *s = (ksw_slice_t *)arg;
    int64_t i, tot = 0;
    for (i = s->lo; i < s->hi; ++i) {
        const orc_job_t *jb = &s->jobs[i];
        int32_t *o = &s->out[i * 6];
        int64_t c = 0;
        o[0] = orc_ksw_extend2(jb->qlen, s->seq + jb->qoff, jb->tlen, s->seq + jb->toff, s->mat,
                               s->o_del, s->e_del, s->o_ins, s->e_ins, jb->w, jb->end_bonus,
                               s->zdrop, jb->h0, &o[1], &o[2], &o[3], &o[4], &o[5], &c);
        if (s->cells) s->cells[i] = c;
        tot += c;
    }
    s->total = tot;
    return 0;
}

int64_t orc_ksw_batch(int64_t n, const void *jobs, const uint8_t *seq,
                      const int8_t mat[25], int o_del, int e_del, int o_ins, int e_ins,
                      int zdrop, int32_t *out, int64_t *cells, int n_threads)
{
    int t;
    int64_t tot = 0;
    ksw_slice_t *sl;
    pthread_t *th;
    if (n_threads < 1) n_threads = 1;
    sl = (ksw_slice_t *)calloc(n_threads, sizeof(ksw_slice_t));
    th = (pthread_t *)calloc(n_threads, sizeof(pthread_t));
    for (t = 0; t < n_threads; ++t) {
        /* interleaved slices would balance better; contiguous slices keep the
         * per-thread memory walk sequential, and the jobs are shuffled anyway */
        sl[t].lo = n * t / n_threads; sl[t].hi = n * (t + 1) / n_threads;
        sl[t].jobs = (const orc_job_t *)jobs; sl[t].seq = seq; sl[t].mat = mat;
        sl[t].o_del = o_del; sl[t].e_del = e_del; sl[t].o_ins = o_ins; sl[t].e_ins = e_ins;
        sl[t].zdrop = zdrop; sl[t].out = out; sl[t].cells = cells;
        if (n_threads == 1) ksw_slice_run(&sl[t]);
        else pthread_create(&th[t], 0, ksw_slice_run, &sl[t]);
    }
    for (t = 0; t < n_threads; ++t) {
        if (n_threads > 1) pthread_join(th[t], 0);
        tot += sl[t].total;
    }
    free(sl); free(th);
    return tot;
}

/* ======================================================================== */
/* FM-index -- bsbolt/External/BWA/bwt.c, bwt.h                             */
/* ======================================================================== */

void orc_bwt_init(orc_bwt_t *b, uint64_t primary, const uint64_t L2_1to4[4],
                  const uint32_t *bwt, uint64_t bwt_size,
                  const uint64_t *sa, uint64_t n_sa, int sa_intv)
{
    memset(b, 0, sizeof(*b));
    b->primary = primary;
    b->L2[0] = 0;
    memcpy(b->L2 + 1, L2_1to4, 4 * sizeof(uint64_t));
    b->seq_len = b->L2[4];            /* bwt.c:454 */
    b->bwt = bwt; b->bwt_size = bwt_size;
    b->sa = sa; b->n_sa = n_sa; b->sa_intv = sa_intv;
}

/* number of 2-bit symbols equal to c among the first n (MSB-first) of word w */
static inline unsigned sym_count(uint32_t w, int c, int n)
{
    uint32_t x = w ^ (0x55555555u * (uint32_t)c);       /* 00 where symbol == c */
    uint32_t hit = ~(x | (x >> 1)) & 0x55555555u;       /* low bit of each matching pair */
    if (n < 16) hit &= ~(0xffffffffu >> (2 * n));        /* keep the first n symbols */
    return (unsigned)__builtin_popcount(hit);
}

/*
 * Occurrence counts of the four bases in rows [0, k] of the $-free BWT
 * (bwt_occ4, bwt.c:169-187).  Block layout (bwt.h:70-73, bwtindex.c:151-173):
 * every 128 symbols, 4 x uint64 cumulative counts then 8 uint32 words of
 * 2-bit symbols, MSB first.  k == (uint64_t)-1 gives all zeros.
 */
void orc_bwt_occ4(const orc_bwt_t *b, uint64_t k, uint64_t cnt[4])
{
    const uint32_t *blk, *w;
    int c, wi, last;
    if (k == (uint64_t)-1) { cnt[0] = cnt[1] = cnt[2] = cnt[3] = 0; return; }
    k -= (k >= b->primary);                      /* the $ row is not stored */
    blk = b->bwt + ((k >> 7) << 4);
    memcpy(cnt, blk, 4 * sizeof(uint64_t));
    w = blk + 8;
    last = (int)((k & 127) >> 4);
    for (c = 0; c < 4; ++c) {
        uint64_t add = 0;
        for (wi = 0; wi < last; ++wi) add += sym_count(w[wi], c, 16);
        add += sym_count(w[last], c, (int)(k & 15) + 1);
        cnt[c] += add;
    }
}

/* bwt_2occ4 (bwt.c:189-220): the same counts at k and l; the reference only
 * shares the block fetch when both fall in one 128-symbol bucket. */
void orc_bwt_2occ4(const orc_bwt_t *b, uint64_t k, uint64_t l, uint64_t ck[4], uint64_t cl[4])
{
    orc_bwt_occ4(b, k, ck);
    orc_bwt_occ4(b, l, cl);
}

/* Bidirectional extension of a bi-interval by all four bases
 * (bwt_extend, bwt.c:262-275).  is_back=1 extends backwards (prepends). */
void orc_bwt_extend(const orc_bwt_t *b, const orc_intv_t *ik, orc_intv_t ok[4], int is_back)
{
    uint64_t tk[4], tl[4];
    int i, f = !is_back;
    orc_bwt_2occ4(b, ik->x[f] - 1, ik->x[f] - 1 + ik->x[2], tk, tl);
    for (i = 0; i < 4; ++i) {
        ok[i].x[f] = b->L2[i] + 1 + tk[i];
        ok[i].x[2] = tl[i] - tk[i];
        ok[i].info = 0;
    }
    ok[3].x[is_back] = ik->x[is_back] +
        (ik->x[f] <= b->primary && ik->x[f] + ik->x[2] - 1 >= b->primary);
    ok[2].x[is_back] = ok[3].x[is_back] + ok[3].x[2];
    ok[1].x[is_back] = ok[2].x[is_back] + ok[2].x[2];
    ok[0].x[is_back] = ok[1].x[is_back] + ok[1].x[2];
}

static inline void set_intv(const orc_bwt_t *b, int c, orc_intv_t *ik)   /* bwt.h:80 */
{
    ik->x[0] = b->L2[c] + 1;
    ik->x[2] = b->L2[c + 1] - b->L2[c];
    ik->x[1] = b->L2[3 - c] + 1;
    ik->info = 0;
}

/* one LF step (bwt_invPsi, bwt.c:53-59, with bwt_occ, bwt.c:109-130) */
static inline uint64_t lf_step(const orc_bwt_t *b, uint64_t k)
{
    uint64_t x, cnt[4], r;
    int c;
    if (k == b->primary) return 0;
    x = k - (k > b->primary);
    c = (int)(b->bwt[((x >> 7) << 4) + 8 + ((x & 127) >> 4)] >> ((~x & 15) << 1) & 3);
    orc_bwt_occ4(b, k, cnt);          /* k < seq_len here, so occ4 == bwt_occ */
    r = b->L2[c] + cnt[c];
    return r;
}

/* bwt_sa (bwt.c:86-96) */
uint64_t orc_bwt_sa(const orc_bwt_t *b, uint64_t k)
{
    uint64_t steps = 0, mask = (uint64_t)b->sa_intv - 1;
    while (k & mask) { ++steps; k = lf_step(b, k); }
    return steps + b->sa[k / (uint64_t)b->sa_intv];
}

/* bwt_smem1 == bwt_smem1a with max_intv = 0 (bwt.c:289-356). */
int orc_bwt_smem1(const orc_bwt_t *b, int len, const uint8_t *q, int x, int min_intv,
                  orc_intv_t *mem, int *n_mem, int max_mem)
{
    orc_intv_t ik, ok[4];
    orc_intv_t *lst0, *lst1, *prev, *curr, *sw;
    int i, j, c, n_prev, n_curr, ret, nm = 0;

    *n_mem = 0;
    if (q[x] > 3) return x + 1;
    if (min_intv < 1) min_intv = 1;
    lst0 = (orc_intv_t *)malloc(sizeof(orc_intv_t) * (len + 2));
    lst1 = (orc_intv_t *)malloc(sizeof(orc_intv_t) * (len + 2));
    curr = lst0; prev = lst1;

    /* forward: remember the interval each time its size is about to change */
    set_intv(b, q[x], &ik);
    ik.info = x + 1;
    n_curr = 0;
    for (i = x + 1; i < len; ++i) {
        if (q[i] < 4) {
            c = 3 - q[i];
            orc_bwt_extend(b, &ik, ok, 0);
            if (ok[c].x[2] != ik.x[2]) {
                curr[n_curr++] = ik;
                if (ok[c].x[2] < (uint64_t)min_intv) break;
            }
            ik = ok[c]; ik.info = i + 1;
        } else {
            curr[n_curr++] = ik;
            break;
        }
    }
    if (i == len) curr[n_curr++] = ik;
    for (j = 0; j < n_curr / 2; ++j) { orc_intv_t t = curr[j]; curr[j] = curr[n_curr - 1 - j]; curr[n_curr - 1 - j] = t; }
    ret = (int)curr[0].info;
    sw = curr; curr = prev; prev = sw;
    n_prev = n_curr;

    /* backward: grow every remembered interval to the left */
    for (i = x - 1; i >= -1; --i) {
        c = i < 0 ? -1 : q[i] < 4 ? q[i] : -1;
        n_curr = 0;
        for (j = 0; j < n_prev; ++j) {
            orc_intv_t *p = &prev[j];
            if (c >= 0) orc_bwt_extend(b, p, ok, 1);
            if (c < 0 || ok[c].x[2] < (uint64_t)min_intv) {
                if (n_curr == 0) {     /* nothing longer survives: p is maximal */
                    if (nm == 0 || (uint64_t)(i + 1) < mem[nm - 1].info >> 32) {
                        if (nm < max_mem) {
                            mem[nm] = *p;
                            mem[nm].info |= (uint64_t)(i + 1) << 32;
                        }
                        ++nm;
                    }
                }
            } else if (n_curr == 0 || ok[c].x[2] != curr[n_curr - 1].x[2]) {
                ok[c].info = p->info;
                curr[n_curr++] = ok[c];
            }
        }
        if (n_curr == 0) break;
        sw = curr; curr = prev; prev = sw;
        n_prev = n_curr;
    }
    if (nm <= max_mem)
        for (j = 0; j < nm / 2; ++j) { orc_intv_t t = mem[j]; mem[j] = mem[nm - 1 - j]; mem[nm - 1 - j] = t; }
    *n_mem = nm;
    free(lst0); free(lst1);
    return ret;
}

/* bwt_seed_strategy1 (bwt.c:358-379) */
int orc_bwt_seed_strategy1(const orc_bwt_t *b, int len, const uint8_t *q, int x,
                           int min_len, int max_intv, orc_intv_t *mem)
{
    orc_intv_t ik, ok[4];
    int i, c;
    memset(mem, 0, sizeof(*mem));
    if (q[x] > 3) return x + 1;
    set_intv(b, q[x], &ik);
    for (i = x + 1; i < len; ++i) {
        if (q[i] < 4) {
            c = 3 - q[i];
            orc_bwt_extend(b, &ik, ok, 0);
            if (ok[c].x[2] < (uint64_t)max_intv && i - x >= min_len) {
                *mem = ok[c];
                mem->info = (uint64_t)x << 32 | (uint64_t)(i + 1);
                return i + 1;
            }
            ik = ok[c];
        } else return i + 1;
    }
    return len;
}

static int intv_cmp(const void *a, const void *b)
{
    uint64_t x = ((const orc_intv_t *)a)->info, y = ((const orc_intv_t *)b)->info;
    return x < y ? -1 : x > y ? 1 : 0;
}

/*
 * mem_collect_intv (bwamem.c:118-166): SMEMs of length >= k, re-seeding
 * inside long SMEMs with few hits, then the LAST-like third pass; sorted by
 * info.  Elements with equal info are the same substring and so the same
 * interval, which makes any correct sort give the reference's order.
 */
int orc_collect_intv(const orc_bwt_t *b, const orc_seed_opt_t *opt, int len, const uint8_t *seq,
                     orc_intv_t *out, int max_out)
{
    int i, k, x = 0, n = 0, old_n, nm;
    int split_len = (int)(opt->min_seed_len * opt->split_factor + .499);
    orc_intv_t *tmp = (orc_intv_t *)malloc(sizeof(orc_intv_t) * (len + 2));
    /* pass 1 */
    while (x < len) {
        if (seq[x] < 4) {
            x = orc_bwt_smem1(b, len, seq, x, 1, tmp, &nm, len + 2);
            for (i = 0; i < nm; ++i) {
                int slen = (int)((uint32_t)tmp[i].info - (uint32_t)(tmp[i].info >> 32));
                if (slen >= opt->min_seed_len) { if (n < max_out) out[n] = tmp[i]; ++n; }
            }
        } else ++x;
    }
    /* pass 2: re-seed in the middle of long, rare SMEMs */
    old_n = n < max_out ? n : max_out;
    for (k = 0; k < old_n; ++k) {
        int start = (int)(out[k].info >> 32), end = (int32_t)out[k].info;
        uint64_t sz = out[k].x[2];
        if (end - start < split_len || sz > (uint64_t)opt->split_width) continue;
        orc_bwt_smem1(b, len, seq, (start + end) >> 1, (int)sz + 1, tmp, &nm, len + 2);
        for (i = 0; i < nm; ++i)
            if ((int)((uint32_t)tmp[i].info - (uint32_t)(tmp[i].info >> 32)) >= opt->min_seed_len) {
                if (n < max_out) out[n] = tmp[i];
                ++n;
            }
    }
    /* pass 3: LAST-like seeds */
    if (opt->max_mem_intv > 0) {
        x = 0;
        while (x < len) {
            if (seq[x] < 4) {
                orc_intv_t m;
                x = orc_bwt_seed_strategy1(b, len, seq, x, opt->min_seed_len, opt->max_mem_intv, &m);
                if (m.x[2] > 0) { if (n < max_out) out[n] = m; ++n; }
            } else ++x;
        }
    }
    free(tmp);
    if (n > max_out) return -1;
    qsort(out, n, sizeof(orc_intv_t), intv_cmp);
    return n;
}

typedef struct {
    const orc_bwt_t *b;
    const orc_seed_opt_t *opt;
    const uint8_t *seqs;
    const int64_t *offs;
    int lo, hi;
    orc_intv_t *buf;     /* per-read scratch, compacted by the caller */
    int *cnt;
    int cap;
} seed_slice_t;

static void *seed_slice_run(void *arg)
{
    seed_slice_t *s = (seed_slice_t *)arg;
    int r;
    for (r = s->lo; r < s->hi; ++r) {
        int len = (int)(s->offs[r + 1] - s->offs[r]);
        s->cnt[r] = orc_collect_intv(s->b, s->opt, len, s->seqs + s->offs[r],
                                     s->buf + (int64_t)r * s->cap, s->cap);
    }
    return 0;
}

int orc_collect_intv_batch(const orc_bwt_t *b, const orc_seed_opt_t *opt, int n,
                           const uint8_t *seqs, const int64_t *offs,
                           orc_intv_t *out, int64_t max_out, int64_t *out_off, int n_threads)
{
    int r, t, maxlen = 0, cap;
    int *cnt;
    orc_intv_t *buf;
    pthread_t *th;
    seed_slice_t *sl;
    int64_t tot = 0;
    for (r = 0; r < n; ++r) {
        int l = (int)(offs[r + 1] - offs[r]);
        if (l > maxlen) maxlen = l;
    }
    cap = 4 * maxlen + 16;   /* each pass adds at most ~len seeds per read */
    cnt = (int *)calloc(n ? n : 1, sizeof(int));
    buf = (orc_intv_t *)malloc(sizeof(orc_intv_t) * (size_t)cap * (n ? n : 1));
    if (n_threads < 1) n_threads = 1;
    th = (pthread_t *)calloc(n_threads, sizeof(pthread_t));
    sl = (seed_slice_t *)calloc(n_threads, sizeof(seed_slice_t));
    for (t = 0; t < n_threads; ++t) {
        sl[t].b = b; sl[t].opt = opt; sl[t].seqs = seqs; sl[t].offs = offs;
        sl[t].lo = (int)((int64_t)n * t / n_threads); sl[t].hi = (int)((int64_t)n * (t + 1) / n_threads);
        sl[t].buf = buf; sl[t].cnt = cnt; sl[t].cap = cap;
        if (n_threads == 1) seed_slice_run(&sl[t]);
        else pthread_create(&th[t], 0, seed_slice_run, &sl[t]);
    }
    if (n_threads > 1) for (t = 0; t < n_threads; ++t) pthread_join(th[t], 0);
    out_off[0] = 0;
    for (r = 0; r < n; ++r) {
        if (cnt[r] < 0 || tot + cnt[r] > max_out) { tot = -1; break; }
        memcpy(out + tot, buf + (int64_t)r * cap, sizeof(orc_intv_t) * cnt[r]);
        tot += cnt[r];
        out_off[r + 1] = tot;
    }
    free(cnt); free(buf); free(th); free(sl);
    return tot < 0 ? -1 : 0;
}

typedef struct {
    const orc_bwt_t *b;
    const uint64_t *k;
    uint64_t *pos;
    int64_t lo, hi;
} sa_slice_t;

static void *sa_slice_run(void *arg)
{
    sa_slice_t *s = (sa_slice_t *)arg;
    int64_t i;
    for (i = s->lo; i < s->hi; ++i) s->pos[i] = orc_bwt_sa(s->b, s->k[i]);
    return 0;
}

void orc_bwt_sa_batch(const orc_bwt_t *b, int64_t n, const uint64_t *k, uint64_t *pos, int n_threads)
{
    int t;
    pthread_t *th;
    sa_slice_t *sl;
    if (n_threads < 1) n_threads = 1;
    th = (pthread_t *)calloc(n_threads, sizeof(pthread_t));
    sl = (sa_slice_t *)calloc(n_threads, sizeof(sa_slice_t));
    for (t = 0; t < n_threads; ++t) {
        sl[t].b = b; sl[t].k = k; sl[t].pos = pos;
        sl[t].lo = n * t / n_threads; sl[t].hi = n * (t + 1) / n_threads;
        if (n_threads == 1) sa_slice_run(&sl[t]);
        else pthread_create(&th[t], 0, sa_slice_run, &sl[t]);
    }
    if (n_threads > 1) for (t = 0; t < n_threads; ++t) pthread_join(th[t], 0);
    free(th); free(sl);
}
