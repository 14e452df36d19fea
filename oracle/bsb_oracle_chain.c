/*
 * bsb_oracle_chain.c -- CPU oracle, part 2 (test infrastructure only):
 * chaining, chain filtering and chain-to-alignment extension of one read.
 *
 * Restates, in our own code, BSBolt's BWA fork (bsbolt/External/BWA):
 *   mem_chain + test_and_merge   bwamem.c:203-319 (the kbtree of chains, kbtree.h)
 *   mem_chain_weight             bwamem.c:229-250
 *   mem_chain_flt                bwamem.c:331-389 (ks_introsort, ksort.h:146-226)
 *   mem_flt_chained_seeds        bwamem.c:602-619 (with mem_seed_sw, bwamem.c:574-598, on the
 *                                ksw_align2 restatement of bsb_oracle_sw.c)
 *   cal_max_gap, mem_chain2aln   bwamem.c:625-790
 *   bns_pos2rid, bns_intv2rid    bntseq.c:364-394
 * Parity is pinned against the reference's own chains and regions
 * (tests/golden/reads_*.npz).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "bsb_oracle.h"
#include "bsb_oracle_chain.h"
#include "bsb_oracle_sw.h"

/* ------------------------------------------------------------- bns lookups */

static int pos2rid(const orc_bns_t *bns, int64_t pos_f)       /* bntseq.c:364-379 */
{
    int left = 0, mid = 0, right = bns->n_seqs;
    if (pos_f >= bns->l_pac) return -1;
    while (left < right) {
        mid = (left + right) >> 1;
        if (pos_f >= bns->anns[mid].offset) {
            if (mid == bns->n_seqs - 1) break;
            if (pos_f < bns->anns[mid + 1].offset) break;
            left = mid + 1;
        } else right = mid;
    }
    return mid;
}

static inline int64_t depos(const orc_bns_t *bns, int64_t pos, int *is_rev)   /* bntseq.h:88-91 */
{
    return (*is_rev = (pos >= bns->l_pac)) ? (bns->l_pac << 1) - 1 - pos : pos;
}

static int intv2rid(const orc_bns_t *bns, int64_t rb, int64_t re)  /* bntseq.c:381-389 */
{
    int is_rev, rid_b, rid_e;
    if (rb < bns->l_pac && re > bns->l_pac) return -2;
    rid_b = pos2rid(bns, depos(bns, rb, &is_rev));
    rid_e = rb < re ? pos2rid(bns, depos(bns, re - 1, &is_rev)) : rid_b;
    return rid_b == rid_e ? rid_b : -1;
}

/* base at position p of the forward-reverse text (bns_get_seq, bntseq.c:414-434) */
static inline int text_base(const orc_bns_t *bns, int64_t p)
{
    if (p < bns->l_pac) return bns->pac[p >> 2] >> ((~p & 3) << 1) & 3;
    p = (bns->l_pac << 1) - 1 - p;
    return 3 - (bns->pac[p >> 2] >> ((~p & 3) << 1) & 3);
}

/* ------------------------------------------------ chains in a kbtree order */

/* The reference keeps chains in a B-tree keyed by the first seed's position
 * (kbtree.h with KB_DEFAULT_SIZE = 512 bytes and 40-byte keys: t = 5, at
 * most 9 keys per node).  Equal keys can occur; which of them a lookup finds
 * and where a new one lands depends on the tree's shape, so the tree is
 * rebuilt here with the same node size and the same split rules. */
#define BT_T 5
#define BT_MAXK (2 * BT_T - 1)

typedef struct {
    int n, internal;
    int key[BT_MAXK];           /* chain indices */
    int child[BT_MAXK + 1];     /* node indices */
} btnode_t;

typedef struct {
    btnode_t *nodes;
    int n_nodes, m_nodes, root;
    const orc_chain_t *chains;  /* key value = chains[idx].pos */
} btree_t;

static int bt_new(btree_t *b)
{
    if (b->n_nodes == b->m_nodes) {
        b->m_nodes = b->m_nodes ? b->m_nodes * 2 : 16;
        b->nodes = (btnode_t *)realloc(b->nodes, sizeof(btnode_t) * b->m_nodes);
    }
    memset(&b->nodes[b->n_nodes], 0, sizeof(btnode_t));
    return b->n_nodes++;
}

static inline int64_t bt_pos(const btree_t *b, int key) { return b->chains[key].pos; }

/* position of k among a node's keys: lower bound, stepped back unless equal
 * (kbtree.h:116-130); *r = 0 when an equal key was found */
static int bt_find(const btree_t *b, const btnode_t *x, int64_t k, int *r)
{
    int begin = 0, end = x->n, tr;
    if (!r) r = &tr;
    if (x->n == 0) return -1;
    while (begin < end) {
        int mid = (begin + end) >> 1;
        if (bt_pos(b, x->key[mid]) < k) begin = mid + 1;
        else end = mid;
    }
    if (begin == x->n) { *r = 1; return x->n - 1; }
    {
        int64_t kb = bt_pos(b, x->key[begin]);
        *r = k < kb ? -1 : (k > kb ? 1 : 0);
    }
    if (*r < 0) --begin;
    return begin;
}

/* kb_intervalp (kbtree.h:151-166): the closest key <= k, or the first equal one met */
static int bt_lower(const btree_t *b, int64_t k)
{
    int lower = -1, xi = b->root;
    while (xi >= 0) {
        const btnode_t *x = &b->nodes[xi];
        int r = 0, i = bt_find(b, x, k, &r);
        if (i >= 0 && r == 0) return x->key[i];
        if (i >= 0) lower = x->key[i];
        if (!x->internal) return lower;
        xi = x->child[i + 1];
    }
    return lower;
}

static void bt_split(btree_t *b, int xi, int i, int yi)       /* kbtree.h:173-190 */
{
    int zi = bt_new(b);
    btnode_t *x = &b->nodes[xi], *y = &b->nodes[yi], *z = &b->nodes[zi];
    int j;
    z->internal = y->internal;
    z->n = BT_T - 1;
    for (j = 0; j < BT_T - 1; ++j) z->key[j] = y->key[BT_T + j];
    if (y->internal)
        for (j = 0; j < BT_T; ++j) z->child[j] = y->child[BT_T + j];
    y->n = BT_T - 1;
    for (j = x->n; j >= i + 1; --j) x->child[j + 1] = x->child[j];
    x->child[i + 1] = zi;
    for (j = x->n - 1; j >= i; --j) x->key[j + 1] = x->key[j];
    x->key[i] = y->key[BT_T - 1];
    ++x->n;
}

static void bt_insert_nonfull(btree_t *b, int xi, int key)    /* kbtree.h:191-209 */
{
    int64_t k = bt_pos(b, key);
    for (;;) {
        btnode_t *x = &b->nodes[xi];
        if (!x->internal) {
            int i = bt_find(b, x, k, 0), j;
            for (j = x->n - 1; j > i; --j) x->key[j + 1] = x->key[j];
            x->key[i + 1] = key;
            ++x->n;
            return;
        } else {
            int i = bt_find(b, x, k, 0) + 1;
            if (b->nodes[x->child[i]].n == BT_MAXK) {
                bt_split(b, xi, i, x->child[i]);
                x = &b->nodes[xi];
                if (k > bt_pos(b, x->key[i])) ++i;
            }
            xi = x->child[i];
        }
    }
}

static void bt_insert(btree_t *b, int key)                    /* kbtree.h:210-223 */
{
    if (b->nodes[b->root].n == BT_MAXK) {
        int si = bt_new(b);
        btnode_t *s = &b->nodes[si];
        s->internal = 1;
        s->n = 0;
        s->child[0] = b->root;
        b->root = si;
        bt_split(b, si, 0, s->child[0]);
    }
    bt_insert_nonfull(b, b->root, key);
}

static void bt_inorder(const btree_t *b, int xi, int *out, int *n)   /* __kb_traverse */
{
    const btnode_t *x = &b->nodes[xi];
    int i;
    for (i = 0; i <= x->n; ++i) {
        if (x->internal) bt_inorder(b, x->child[i], out, n);
        if (i < x->n) out[(*n)++] = x->key[i];
    }
}

/* -------------------------------------------------------------- mem_chain */

typedef struct {
    orc_seed_t *a;
    int n, m;
} seedvec_t;

/* test_and_merge (bwamem.c:203-227) */
static int test_and_merge(const orc_opt_t *opt, int64_t l_pac, orc_chain_t *c, seedvec_t *sv,
                          const orc_seed_t *p, int seed_rid)
{
    const orc_seed_t *first = &sv->a[0], *last = &sv->a[sv->n - 1];
    int64_t qend = last->qbeg + last->len, rend = last->rbeg + last->len, x, y;
    if (seed_rid != c->rid) return 0;
    if (p->qbeg >= first->qbeg && p->qbeg + p->len <= qend && p->rbeg >= first->rbeg && p->rbeg + p->len <= rend)
        return 1;
    if ((last->rbeg < l_pac || first->rbeg < l_pac) && p->rbeg >= l_pac) return 0;
    x = p->qbeg - last->qbeg;
    y = p->rbeg - last->rbeg;
    if (y >= 0 && x - y <= opt->w && y - x <= opt->w && x - last->len < opt->max_chain_gap &&
        y - last->len < opt->max_chain_gap) {
        if (sv->n == sv->m) {
            sv->m <<= 1;
            sv->a = (orc_seed_t *)realloc(sv->a, sizeof(orc_seed_t) * sv->m);
        }
        sv->a[sv->n++] = *p;
        c->n = sv->n;
        return 1;
    }
    return 0;
}

int orc_mem_chain(const orc_bwt_t *bwt, const orc_bns_t *bns, const orc_opt_t *opt, int len,
                  const orc_intv_t *mem, int n_mem, orc_chain_t **chains_out, orc_seed_t **seeds_out,
                  int *n_seeds_out)
{
    int i, b = 0, e = 0, l_rep = 0, n_chn = 0, m_chn = 16, n_order = 0, k;
    orc_chain_t *chn;
    seedvec_t *sv;
    btree_t bt;
    int *order;
    orc_seed_t *seeds;
    int total = 0;

    *chains_out = NULL; *seeds_out = NULL; *n_seeds_out = 0;
    if (len < opt->min_seed_len) return 0;     /* bwamem.c:266 */
    /* fraction of the read covered by repetitive seeds (bwamem.c:271-278) */
    for (i = 0; i < n_mem; ++i) {
        int sb = (int)(mem[i].info >> 32), se = (int)(uint32_t)mem[i].info;
        if (mem[i].x[2] <= (uint64_t)opt->max_occ) continue;
        if (sb > e) l_rep += e - b, b = sb, e = se;
        else e = e > se ? e : se;
    }
    l_rep += e - b;

    chn = (orc_chain_t *)calloc(m_chn, sizeof(orc_chain_t));
    sv = (seedvec_t *)calloc(m_chn, sizeof(seedvec_t));
    memset(&bt, 0, sizeof bt);
    bt.chains = chn;
    bt.root = bt_new(&bt);
    for (i = 0; i < n_mem; ++i) {
        const orc_intv_t *p = &mem[i];
        int slen = (int)((uint32_t)p->info - (uint32_t)(p->info >> 32));
        int64_t kk, count;
        uint64_t step = p->x[2] > (uint64_t)opt->max_occ ? p->x[2] / (uint64_t)opt->max_occ : 1;
        for (kk = count = 0; (uint64_t)kk < p->x[2] && count < opt->max_occ; kk += (int64_t)step, ++count) {
            orc_seed_t s;
            int rid, to_add = 0;
            s.rbeg = (int64_t)orc_bwt_sa(bwt, p->x[0] + (uint64_t)kk);
            s.qbeg = (int32_t)(p->info >> 32);
            s.score = s.len = slen;
            rid = intv2rid(bns, s.rbeg, s.rbeg + s.len);
            if (rid < 0) continue;
            if (n_chn > 0) {
                int lower = bt_lower(&bt, s.rbeg);
                if (lower < 0 || !test_and_merge(opt, bns->l_pac, &chn[lower], &sv[lower], &s, rid)) to_add = 1;
            } else to_add = 1;
            if (to_add) {
                if (n_chn == m_chn) {
                    m_chn <<= 1;
                    chn = (orc_chain_t *)realloc(chn, sizeof(orc_chain_t) * m_chn);
                    sv = (seedvec_t *)realloc(sv, sizeof(seedvec_t) * m_chn);
                    bt.chains = chn;
                }
                memset(&chn[n_chn], 0, sizeof(orc_chain_t));
                chn[n_chn].n = 1;
                chn[n_chn].rid = rid;
                chn[n_chn].is_alt = 0;
                chn[n_chn].pos = s.rbeg;
                sv[n_chn].m = 4;
                sv[n_chn].n = 1;
                sv[n_chn].a = (orc_seed_t *)calloc(4, sizeof(orc_seed_t));
                sv[n_chn].a[0] = s;
                bt_insert(&bt, n_chn);
                ++n_chn;
            }
        }
    }
    order = (int *)malloc(sizeof(int) * (n_chn ? n_chn : 1));
    if (n_chn) bt_inorder(&bt, bt.root, order, &n_order);
    for (i = 0; i < n_chn; ++i) total += sv[i].n;
    seeds = (orc_seed_t *)malloc(sizeof(orc_seed_t) * (total ? total : 1));
    {
        orc_chain_t *out = (orc_chain_t *)malloc(sizeof(orc_chain_t) * (n_chn ? n_chn : 1));
        int off = 0;
        for (k = 0; k < n_order; ++k) {
            int c = order[k];
            out[k] = chn[c];
            out[k].n = sv[c].n;
            out[k].seed_off = off;
            out[k].frac_rep = (float)l_rep / len;
            memcpy(seeds + off, sv[c].a, sizeof(orc_seed_t) * sv[c].n);
            off += sv[c].n;
        }
        *chains_out = out;
    }
    for (i = 0; i < n_chn; ++i) free(sv[i].a);
    free(sv); free(chn); free(order); free(bt.nodes);
    *seeds_out = seeds;
    *n_seeds_out = total;
    return n_order;
}

/* mem_chain_weight (bwamem.c:229-250) */
static int chain_weight(const orc_chain_t *c, const orc_seed_t *seeds)
{
    int64_t end;
    int j, w = 0, tmp;
    const orc_seed_t *s = seeds + c->seed_off;
    for (j = 0, end = 0; j < c->n; ++j) {
        if (s[j].qbeg >= end) w += s[j].len;
        else if (s[j].qbeg + s[j].len > end) w += (int)(s[j].qbeg + s[j].len - end);
        end = end > s[j].qbeg + s[j].len ? end : s[j].qbeg + s[j].len;
    }
    tmp = w; w = 0;
    for (j = 0, end = 0; j < c->n; ++j) {
        if (s[j].rbeg >= end) w += s[j].len;
        else if (s[j].rbeg + s[j].len > end) w += (int)(s[j].rbeg + s[j].len - end);
        end = end > s[j].rbeg + s[j].len ? end : s[j].rbeg + s[j].len;
    }
    w = w < tmp ? w : tmp;
    return w < 1 << 30 ? w : (1 << 30) - 1;
}

/* ks_introsort with the comparison a.w > b.w (ksort.h:146-226, bwamem.c:328-329),
 * restated step for step because chains of equal weight keep the order it leaves. */
#define FLT_LT(a, b) ((a).w > (b).w)

static void flt_insertsort(orc_chain_t *s, orc_chain_t *t)
{
    orc_chain_t *i, *j, tmp;
    for (i = s + 1; i < t; ++i)
        for (j = i; j > s && FLT_LT(*j, *(j - 1)); --j) { tmp = *j; *j = *(j - 1); *(j - 1) = tmp; }
}

static void flt_combsort(size_t n, orc_chain_t *a)
{
    const double shrink_factor = 1.2473309501039786540366528676643;
    int do_swap;
    size_t gap = n;
    orc_chain_t tmp, *i, *j;
    do {
        if (gap > 2) {
            gap = (size_t)(gap / shrink_factor);
            if (gap == 9 || gap == 10) gap = 11;
        }
        do_swap = 0;
        for (i = a; i < a + n - gap; ++i) {
            j = i + gap;
            if (FLT_LT(*j, *i)) { tmp = *i; *i = *j; *j = tmp; do_swap = 1; }
        }
    } while (do_swap || gap > 2);
    if (gap != 1) flt_insertsort(a, a + n);
}

static void flt_introsort(size_t n, orc_chain_t *a)
{
    typedef struct { orc_chain_t *left, *right; int depth; } frame_t;
    int d;
    frame_t *top, *stack;
    orc_chain_t rp, tmp, *s, *t, *i, *j, *k;
    if (n < 1) return;
    if (n == 2) {
        if (FLT_LT(a[1], a[0])) { tmp = a[0]; a[0] = a[1]; a[1] = tmp; }
        return;
    }
    for (d = 2; 1ul << d < n; ++d) ;
    stack = (frame_t *)malloc(sizeof(frame_t) * ((sizeof(size_t) * d) + 2));
    top = stack; s = a; t = a + (n - 1); d <<= 1;
    for (;;) {
        if (s < t) {
            if (--d == 0) {
                flt_combsort(t - s + 1, s);
                t = s;
                continue;
            }
            i = s; j = t; k = i + ((j - i) >> 1) + 1;
            if (FLT_LT(*k, *i)) {
                if (FLT_LT(*k, *j)) k = j;
            } else k = FLT_LT(*j, *i) ? i : j;
            rp = *k;
            if (k != t) { tmp = *k; *k = *t; *t = tmp; }
            for (;;) {
                do ++i; while (FLT_LT(*i, rp));
                do --j; while (i <= j && FLT_LT(rp, *j));
                if (j <= i) break;
                tmp = *i; *i = *j; *j = tmp;
            }
            tmp = *i; *i = *t; *t = tmp;
            if (i - s > t - i) {
                if (i - s > 16) { top->left = s; top->right = i - 1; top->depth = d; ++top; }
                s = t - i > 16 ? i + 1 : t;
            } else {
                if (t - i > 16) { top->left = i + 1; top->right = t; top->depth = d; ++top; }
                t = i - s > 16 ? i - 1 : s;
            }
        } else {
            if (top == stack) {
                free(stack);
                flt_insertsort(a, a + n);
                return;
            } else { --top; s = top->left; t = top->right; d = top->depth; }
        }
    }
}

#define CHN_BEG(c, sd) ((sd)[(c).seed_off].qbeg)
#define CHN_END(c, sd) ((sd)[(c).seed_off + (c).n - 1].qbeg + (sd)[(c).seed_off + (c).n - 1].len)

/* mem_chain_flt (bwamem.c:331-389).  Chains are compacted in place; seed
 * arrays stay where they are (seed_off). */
int orc_mem_chain_flt(const orc_opt_t *opt, int n_chn, orc_chain_t *a, const orc_seed_t *sd)
{
    int i, k, n_kept = 0;
    int *kept_idx;
    if (n_chn == 0) return 0;
    for (i = k = 0; i < n_chn; ++i) {
        orc_chain_t *c = &a[i];
        c->first = -1; c->kept = 0;
        c->w = chain_weight(c, sd);
        if (c->w >= opt->min_chain_weight) a[k++] = *c;
    }
    n_chn = k;
    flt_introsort(n_chn, a);
    kept_idx = (int *)malloc(sizeof(int) * (n_chn ? n_chn : 1));
    a[0].kept = 3;
    kept_idx[n_kept++] = 0;
    for (i = 1; i < n_chn; ++i) {
        int large_ovlp = 0;
        for (k = 0; k < n_kept; ++k) {
            int j = kept_idx[k];
            int b_max = CHN_BEG(a[j], sd) > CHN_BEG(a[i], sd) ? CHN_BEG(a[j], sd) : CHN_BEG(a[i], sd);
            int e_min = CHN_END(a[j], sd) < CHN_END(a[i], sd) ? CHN_END(a[j], sd) : CHN_END(a[i], sd);
            if (e_min > b_max && (!a[j].is_alt || a[i].is_alt)) {
                int li = CHN_END(a[i], sd) - CHN_BEG(a[i], sd);
                int lj = CHN_END(a[j], sd) - CHN_BEG(a[j], sd);
                int min_l = li < lj ? li : lj;
                if (e_min - b_max >= min_l * opt->mask_level && min_l < opt->max_chain_gap) {
                    large_ovlp = 1;
                    if (a[j].first < 0) a[j].first = i;
                    if (a[i].w < a[j].w * opt->drop_ratio && a[j].w - a[i].w >= opt->min_seed_len << 1) break;
                }
            }
        }
        if (k == n_kept) {
            kept_idx[n_kept++] = i;
            a[i].kept = large_ovlp ? 2 : 3;
        }
    }
    for (i = 0; i < n_kept; ++i) {
        orc_chain_t *c = &a[kept_idx[i]];
        if (c->first >= 0) a[c->first].kept = 1;
    }
    free(kept_idx);
    for (i = k = 0; i < n_chn; ++i) {
        if (a[i].kept == 0 || a[i].kept == 3) continue;
        if (++k >= opt->max_chain_extend) break;
    }
    for (; i < n_chn; ++i)
        if (a[i].kept < 3) a[i].kept = 0;
    for (i = k = 0; i < n_chn; ++i)
        if (a[i].kept != 0) a[k++] = a[i];
    return k;
}

/* mem_flt_chained_seeds (bwamem.c:602-619) returns at once for these read
 * lengths; returns 1 if the seed-level SW filter would run (not restated). */
int orc_seed_sw_filter_applies(const orc_opt_t *opt, int l_query)
{
    double min_l = opt->min_chain_weight ? 1.1f * opt->min_chain_weight : 5.5f * log(l_query);
    return !(min_l > 0.05f * l_query);
}

/* mem_seed_sw (bwamem.c:574-598): the best local score of the seed's neighbourhood, 50 bases
 * each side, or -1 when the seed or the window is long enough to need none. */
static int orc_mem_seed_sw(const orc_opt_t *opt, const orc_bns_t *bns, int l_query, const uint8_t *query,
                           const orc_seed_t *s)
{
    int qb, qe, is_rev, rid, score;
    int64_t rb, re, mid, l_pac = bns->l_pac, far_beg, far_end, k;
    uint8_t *rseq;
    orc_kswr_t x;
    if (s->len >= 200) return -1;                               /* MEM_SHORT_LEN */
    qb = s->qbeg, qe = s->qbeg + s->len;
    rb = s->rbeg, re = s->rbeg + s->len;
    mid = (rb + re) >> 1;
    qb -= 50; qb = qb > 0 ? qb : 0;                             /* MEM_SHORT_EXT */
    qe += 50; qe = qe < l_query ? qe : l_query;
    rb -= 50; rb = rb > 0 ? rb : 0;
    re += 50; re = re < l_pac << 1 ? re : l_pac << 1;
    if (rb < l_pac && l_pac < re) {
        if (mid < l_pac) re = l_pac;
        else rb = l_pac;
    }
    if (qe - qb >= 200 || re - rb >= 200) return -1;
    /* bns_fetch_seq (bntseq.c:436-461): the window clipped to the contig of its middle */
    rid = pos2rid(bns, depos(bns, mid, &is_rev));
    far_beg = bns->anns[rid].offset;
    far_end = far_beg + bns->anns[rid].len;
    if (is_rev) {
        int64_t t = far_beg;
        far_beg = (l_pac << 1) - far_end;
        far_end = (l_pac << 1) - t;
    }
    rb = rb > far_beg ? rb : far_beg;
    re = re < far_end ? re : far_end;
    rseq = (uint8_t *)malloc((size_t)(re - rb) + 1);
    for (k = rb; k < re; ++k) rseq[k - rb] = (uint8_t)text_base(bns, k);
    x = orc_ksw_align2(qe - qb, query + qb, (int)(re - rb), rseq, opt->mat, opt->o_del, opt->e_del, opt->o_ins,
                       opt->e_ins, ORC_KSW_XSTART);
    score = x.score;
    free(rseq);
    return score;
}

/* mem_flt_chained_seeds (bwamem.c:602-619): each chain keeps, in order, the seeds whose
 * neighbourhood scores at least min_HSP_score or that need no SW, rescored; a no-op for
 * read lengths where the reference returns early. */
void orc_flt_chained_seeds(const orc_opt_t *opt, const orc_bns_t *bns, int l_query, const uint8_t *query,
                           int n_chn, orc_chain_t *a, orc_seed_t *seeds)
{
    double min_l = opt->min_chain_weight ? 1.1f * opt->min_chain_weight : 5.5f * log(l_query);
    int i, j, k, min_HSP_score = (int)(opt->a * min_l + .499);
    if (min_l > 0.05f * l_query) return;
    for (i = 0; i < n_chn; ++i) {
        orc_chain_t *c = &a[i];
        orc_seed_t *cs = seeds + c->seed_off;
        for (j = k = 0; j < c->n; ++j) {
            orc_seed_t sd = cs[j];
            sd.score = orc_mem_seed_sw(opt, bns, l_query, query, &sd);
            if (sd.score < 0 || sd.score >= min_HSP_score) {
                sd.score = sd.score < 0 ? sd.len * opt->a : sd.score;
                cs[k++] = sd;
            }
        }
        c->n = k;
    }
}

/* cal_max_gap (bwamem.c:625-632) */
static inline int cal_max_gap(const orc_opt_t *opt, int qlen)
{
    int l_del = (int)((double)(qlen * opt->a - opt->o_del) / opt->e_del + 1.);
    int l_ins = (int)((double)(qlen * opt->a - opt->o_ins) / opt->e_ins + 1.);
    int l = l_del > l_ins ? l_del : l_ins;
    l = l > 1 ? l : 1;
    return l < opt->w << 1 ? l : opt->w << 1;
}

static int u64_cmp(const void *x, const void *y)
{
    uint64_t a = *(const uint64_t *)x, b = *(const uint64_t *)y;
    return a < b ? -1 : a > b;
}

/* mem_chain2aln (bwamem.c:636-790): appends to regs[*n_regs] (capacity max_regs). */
int orc_mem_chain2aln(const orc_opt_t *opt, const orc_bns_t *bns, int l_query, const uint8_t *query,
                      const orc_chain_t *c, const orc_seed_t *sd, orc_reg_t *regs, int *n_regs, int max_regs,
                      int64_t *cells)
{
    int i, k, rid = -1, max_off[2], aw[2];
    int64_t l_pac = bns->l_pac, rmax[2], tmp, mx = 0;
    const orc_seed_t *seeds = sd + c->seed_off, *s;
    uint64_t *srt;
    uint8_t *rseq;

    if (c->n == 0) return 0;
    rmax[0] = l_pac << 1; rmax[1] = 0;
    for (i = 0; i < c->n; ++i) {
        int64_t b, e;
        const orc_seed_t *t = &seeds[i];
        b = t->rbeg - (t->qbeg + cal_max_gap(opt, t->qbeg));
        e = t->rbeg + t->len + ((l_query - t->qbeg - t->len) + cal_max_gap(opt, l_query - t->qbeg - t->len));
        rmax[0] = rmax[0] < b ? rmax[0] : b;
        rmax[1] = rmax[1] > e ? rmax[1] : e;
        if (t->len > mx) mx = t->len;
    }
    rmax[0] = rmax[0] > 0 ? rmax[0] : 0;
    rmax[1] = rmax[1] < l_pac << 1 ? rmax[1] : l_pac << 1;
    if (rmax[0] < l_pac && l_pac < rmax[1]) {
        if (seeds[0].rbeg < l_pac) rmax[1] = l_pac;
        else rmax[0] = l_pac;
    }
    /* bns_fetch_seq (bntseq.c:436-461): clip the window to the seed's contig */
    {
        int is_rev;
        int64_t far_beg, far_end, mid = seeds[0].rbeg;
        rid = pos2rid(bns, depos(bns, mid, &is_rev));
        far_beg = bns->anns[rid].offset;
        far_end = far_beg + bns->anns[rid].len;
        if (is_rev) {
            int64_t t = far_beg;
            far_beg = (l_pac << 1) - far_end;
            far_end = (l_pac << 1) - t;
        }
        rmax[0] = rmax[0] > far_beg ? rmax[0] : far_beg;
        rmax[1] = rmax[1] < far_end ? rmax[1] : far_end;
        if (rid != c->rid) return -2;
    }
    rseq = (uint8_t *)malloc((size_t)(rmax[1] - rmax[0]) + 1);
    for (tmp = rmax[0]; tmp < rmax[1]; ++tmp) rseq[tmp - rmax[0]] = (uint8_t)text_base(bns, tmp);

    srt = (uint64_t *)malloc(8 * (size_t)c->n);
    for (i = 0; i < c->n; ++i) srt[i] = (uint64_t)seeds[i].score << 32 | (uint32_t)i;
    qsort(srt, c->n, 8, u64_cmp);   /* keys are distinct, so any sort gives ks_introsort_64's order */

    for (k = c->n - 1; k >= 0; --k) {
        orc_reg_t *a;
        s = &seeds[(uint32_t)srt[k]];
        for (i = 0; i < *n_regs; ++i) {          /* is the seed (almost) inside an earlier hit? */
            const orc_reg_t *p = &regs[i];
            int64_t rd;
            int qd, w, max_gap;
            if (s->rbeg < p->rb || s->rbeg + s->len > p->re || s->qbeg < p->qb || s->qbeg + s->len > p->qe) continue;
            if (s->len - p->seedlen0 > .1 * l_query) continue;
            qd = s->qbeg - p->qb; rd = s->rbeg - p->rb;
            max_gap = cal_max_gap(opt, qd < rd ? qd : (int)rd);
            w = max_gap < p->w ? max_gap : p->w;
            if (qd - rd < w && rd - qd < w) break;
            qd = p->qe - (s->qbeg + s->len); rd = p->re - (s->rbeg + s->len);
            max_gap = cal_max_gap(opt, qd < rd ? qd : (int)rd);
            w = max_gap < p->w ? max_gap : p->w;
            if (qd - rd < w && rd - qd < w) break;
        }
        if (i < *n_regs) {
            for (i = k + 1; i < c->n; ++i) {     /* overlapping seeds in the same chain */
                const orc_seed_t *t;
                if (srt[i] == 0) continue;
                t = &seeds[(uint32_t)srt[i]];
                if (t->len < s->len * .95) continue;
                if (s->qbeg <= t->qbeg && s->qbeg + s->len - t->qbeg >= s->len >> 2 && t->qbeg - s->qbeg != t->rbeg - s->rbeg) break;
                if (t->qbeg <= s->qbeg && t->qbeg + t->len - s->qbeg >= s->len >> 2 && s->qbeg - t->qbeg != s->rbeg - t->rbeg) break;
            }
            if (i == c->n) { srt[k] = 0; continue; }
        }
        if (*n_regs >= max_regs) { free(srt); free(rseq); return -1; }
        a = &regs[(*n_regs)++];
        memset(a, 0, sizeof(*a));
        a->w = aw[0] = aw[1] = opt->w;
        a->score = a->truesc = -1;
        a->rid = c->rid;
        if (s->qbeg) {                           /* left extension on reversed copies */
            uint8_t *rs, *qs;
            int qle, tle, gtle, gscore;
            int64_t cc;
            qs = (uint8_t *)malloc(s->qbeg);
            for (i = 0; i < s->qbeg; ++i) qs[i] = query[s->qbeg - 1 - i];
            tmp = s->rbeg - rmax[0];
            rs = (uint8_t *)malloc((size_t)tmp + 1);
            for (i = 0; i < tmp; ++i) rs[i] = rseq[tmp - 1 - i];
            for (i = 0; i < 2; ++i) {
                int prev = a->score;
                aw[0] = opt->w << i;
                a->score = orc_ksw_extend2(s->qbeg, qs, (int)tmp, rs, opt->mat, opt->o_del, opt->e_del, opt->o_ins,
                                           opt->e_ins, aw[0], opt->pen_clip5, opt->zdrop, s->len * opt->a,
                                           &qle, &tle, &gtle, &gscore, &max_off[0], &cc);
                if (cells) *cells += cc;
                if (a->score == prev || max_off[0] < (aw[0] >> 1) + (aw[0] >> 2)) break;
            }
            if (gscore <= 0 || gscore <= a->score - opt->pen_clip5) {
                a->qb = s->qbeg - qle, a->rb = s->rbeg - tle;
                a->truesc = a->score;
            } else {
                a->qb = 0, a->rb = s->rbeg - gtle;
                a->truesc = gscore;
            }
            free(qs); free(rs);
        } else a->score = a->truesc = s->len * opt->a, a->qb = 0, a->rb = s->rbeg;

        if (s->qbeg + s->len != l_query) {       /* right extension */
            int qle, tle, qe, re, gtle, gscore, sc0 = a->score;
            int64_t cc;
            qe = s->qbeg + s->len;
            re = (int)(s->rbeg + s->len - rmax[0]);
            for (i = 0; i < 2; ++i) {
                int prev = a->score;
                aw[1] = opt->w << i;
                a->score = orc_ksw_extend2(l_query - qe, query + qe, (int)(rmax[1] - rmax[0] - re), rseq + re,
                                           opt->mat, opt->o_del, opt->e_del, opt->o_ins, opt->e_ins, aw[1],
                                           opt->pen_clip3, opt->zdrop, sc0, &qle, &tle, &gtle, &gscore,
                                           &max_off[1], &cc);
                if (cells) *cells += cc;
                if (a->score == prev || max_off[1] < (aw[1] >> 1) + (aw[1] >> 2)) break;
            }
            if (gscore <= 0 || gscore <= a->score - opt->pen_clip3) {
                a->qe = qe + qle, a->re = rmax[0] + re + tle;
                a->truesc += a->score - sc0;
            } else {
                a->qe = l_query, a->re = rmax[0] + re + gtle;
                a->truesc += gscore - sc0;
            }
        } else a->qe = l_query, a->re = s->rbeg + s->len;

        for (i = 0, a->seedcov = 0; i < c->n; ++i) {
            const orc_seed_t *t = &seeds[i];
            if (t->qbeg >= a->qb && t->qbeg + t->len <= a->qe && t->rbeg >= a->rb && t->rbeg + t->len <= a->re)
                a->seedcov += t->len;
        }
        a->w = aw[0] > aw[1] ? aw[0] : aw[1];
        a->seedlen0 = s->len;
        a->frac_rep = c->frac_rep;
    }
    free(srt); free(rseq);
    return 0;
}

/* ------------------------------------------------------------ batch driver */

#include <pthread.h>

typedef struct {
    orc_chain_t *c0; int n0;
    orc_seed_t *s0; int ns;
    orc_chain_t *c1; int n1;
    orc_reg_t *r; int nr;
    int64_t cells;
    int err;
} read_res_t;

typedef struct {
    const orc_bwt_t *bwt;
    const orc_bns_t *bns;
    const orc_opt_t *opt;
    const uint8_t *seqs;
    const int64_t *offs;
    read_res_t *res;
    int lo, hi;
} align_slice_t;

static void align_one(const orc_bwt_t *bwt, const orc_bns_t *bns, const orc_opt_t *opt, int len,
                      const uint8_t *q, read_res_t *rr)
{
    orc_seed_opt_t so;
    orc_intv_t *mem;
    int n_mem, i, max_regs;
    memset(rr, 0, sizeof(*rr));
    so.min_seed_len = opt->min_seed_len; so.split_factor = opt->split_factor;
    so.split_width = opt->split_width; so.max_mem_intv = opt->max_mem_intv;
    mem = (orc_intv_t *)malloc(sizeof(orc_intv_t) * (4 * (size_t)len + 16));
    n_mem = len >= opt->min_seed_len ? orc_collect_intv(bwt, &so, len, q, mem, 4 * len + 16) : 0;
    if (n_mem < 0) { rr->err = -1; free(mem); return; }
    rr->n0 = orc_mem_chain(bwt, bns, opt, len, mem, n_mem, &rr->c0, &rr->s0, &rr->ns);
    free(mem);
    rr->c1 = (orc_chain_t *)malloc(sizeof(orc_chain_t) * (rr->n0 ? rr->n0 : 1));
    memcpy(rr->c1, rr->c0, sizeof(orc_chain_t) * rr->n0);
    rr->n1 = orc_mem_chain_flt(opt, rr->n0, rr->c1, rr->s0);
    /* the filter rewrites the kept chains' seeds in place: the pre-filter chain list (c0)
     * shares those seed ranges and is reported only for reads the filter leaves alone */
    if (rr->n1 > 0) orc_flt_chained_seeds(opt, bns, len, q, rr->n1, rr->c1, rr->s0);
    max_regs = rr->ns + 1;
    rr->r = (orc_reg_t *)malloc(sizeof(orc_reg_t) * max_regs);
    for (i = 0; i < rr->n1; ++i)
        if (orc_mem_chain2aln(opt, bns, len, q, &rr->c1[i], rr->s0, rr->r, &rr->nr, max_regs, &rr->cells) != 0) {
            rr->err = -2;
            return;
        }
}

static void *align_slice_run(void *arg)
{
    align_slice_t *s = (align_slice_t *)arg;
    int r;
    for (r = s->lo; r < s->hi; ++r)
        align_one(s->bwt, s->bns, s->opt, (int)(s->offs[r + 1] - s->offs[r]), s->seqs + s->offs[r], &s->res[r]);
    return 0;
}

int orc_align_regs_batch(const orc_bwt_t *bwt, const orc_bns_t *bns, const orc_opt_t *opt, int n_reads,
                         const uint8_t *seqs, const int64_t *offs, orc_align_out_t *out, int n_threads)
{
    read_res_t *res = (read_res_t *)calloc(n_reads ? n_reads : 1, sizeof(read_res_t));
    pthread_t *th;
    align_slice_t *sl;
    int t, r, err = 0;
    int64_t t0 = 0, ts = 0, t1 = 0, tr = 0;
    if (n_threads < 1) n_threads = 1;
    th = (pthread_t *)calloc(n_threads, sizeof(pthread_t));
    sl = (align_slice_t *)calloc(n_threads, sizeof(align_slice_t));
    for (t = 0; t < n_threads; ++t) {
        sl[t].bwt = bwt; sl[t].bns = bns; sl[t].opt = opt; sl[t].seqs = seqs; sl[t].offs = offs; sl[t].res = res;
        sl[t].lo = (int)((int64_t)n_reads * t / n_threads); sl[t].hi = (int)((int64_t)n_reads * (t + 1) / n_threads);
        if (n_threads == 1) align_slice_run(&sl[t]);
        else pthread_create(&th[t], 0, align_slice_run, &sl[t]);
    }
    if (n_threads > 1) for (t = 0; t < n_threads; ++t) pthread_join(th[t], 0);
    for (r = 0; r < n_reads; ++r) {
        if (res[r].err) err = res[r].err;
        t0 += res[r].n0; ts += res[r].ns; t1 += res[r].n1; tr += res[r].nr;
    }
    memset(out, 0, sizeof(*out));
    out->chain0 = (orc_chain_t *)malloc(sizeof(orc_chain_t) * (t0 + 1));
    out->seeds0 = (orc_seed_t *)malloc(sizeof(orc_seed_t) * (ts + 1));
    out->chain1 = (orc_chain_t *)malloc(sizeof(orc_chain_t) * (t1 + 1));
    out->regs = (orc_reg_t *)malloc(sizeof(orc_reg_t) * (tr + 1));
    out->chain0_off = (int64_t *)calloc(n_reads + 1, 8);
    out->seeds0_off = (int64_t *)calloc(n_reads + 1, 8);
    out->chain1_off = (int64_t *)calloc(n_reads + 1, 8);
    out->regs_off = (int64_t *)calloc(n_reads + 1, 8);
    t0 = ts = t1 = tr = 0;
    for (r = 0; r < n_reads; ++r) {
        read_res_t *x = &res[r];
        memcpy(out->chain0 + t0, x->c0, sizeof(orc_chain_t) * x->n0);
        memcpy(out->seeds0 + ts, x->s0, sizeof(orc_seed_t) * x->ns);
        memcpy(out->chain1 + t1, x->c1, sizeof(orc_chain_t) * x->n1);
        memcpy(out->regs + tr, x->r, sizeof(orc_reg_t) * x->nr);
        t0 += x->n0; ts += x->ns; t1 += x->n1; tr += x->nr;
        out->chain0_off[r + 1] = t0; out->seeds0_off[r + 1] = ts;
        out->chain1_off[r + 1] = t1; out->regs_off[r + 1] = tr;
        out->cells += x->cells;
        free(x->c0); free(x->s0); free(x->c1); free(x->r);
    }
    free(res); free(th); free(sl);
    return err;
}

void orc_align_out_free(orc_align_out_t *o)
{
    free(o->chain0); free(o->seeds0); free(o->chain1); free(o->regs);
    free(o->chain0_off); free(o->seeds0_off); free(o->chain1_off); free(o->regs_off);
}
