/*
 * bsb_oracle_sw.c -- CPU oracle for ksw_align2 (see bsb_oracle_sw.h).
 *
 * TEST INFRASTRUCTURE ONLY.  Restates bsbolt/External/BWA/ksw.c:
 *   ksw_qinit   :48-96   query profile, striped: vector j, lane l holds column j + l*slen
 *   ksw_u8      :98-212  8-bit lanes (16 per vector), scores offset by `shift`, saturating
 *   ksw_i16     :214-327 16-bit lanes (8 per vector), saturating
 *   ksw_align2  :336-360 the forward pass, then the start positions from a second pass
 *                        over the reversed prefixes
 * A vector is an array of P lane values; every SSE2 operation the reference uses
 * (adds/subs with saturation, max, byte/word shifts, movemask tests) is written
 * out per lane.
 */
#include "bsb_oracle_sw.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int size, p, slen, qlen;
    int shift, mdiff, max;          /* as the reference's uint8 fields */
    int16_t *qp;                    /* [5][slen][p] */
} prof_t;

static void qinit(prof_t *q, int size, int qlen, const uint8_t *query, const int8_t mat[25])
{
    q->size = size > 1 ? 2 : 1;
    q->p = 8 * (3 - q->size);
    q->qlen = qlen;
    q->slen = (qlen + q->p - 1) / q->p;
    /* min / max score as the reference finds them with uint8 fields (ksw.c:66-71) */
    uint8_t shift = 127, mdiff = 0;
    for (int a = 0; a < 25; ++a) {
        if (mat[a] < (int8_t)shift) shift = (uint8_t)mat[a];
        if (mat[a] > (int8_t)mdiff) mdiff = (uint8_t)mat[a];
    }
    q->max = mdiff;
    shift = (uint8_t)(256 - shift);
    mdiff = (uint8_t)(mdiff + shift);
    q->shift = shift, q->mdiff = mdiff;
    const int n = q->slen * q->p;
    q->qp = malloc(sizeof(int16_t) * 5 * (n > 0 ? n : 1));
    for (int a = 0; a < 5; ++a)
        for (int j = 0; j < q->slen; ++j)
            for (int l = 0; l < q->p; ++l) {
                const int k = j + l * q->slen;
                int v = k >= qlen ? 0 : mat[a * 5 + query[k]];
                if (q->size == 1) v = (uint8_t)(int8_t)(v + shift);   /* stored as int8, read as uint8 */
                q->qp[(a * q->slen + j) * q->p + l] = (int16_t)v;
            }
}

static inline int sat_u8(int x) { return x < 0 ? 0 : x > 255 ? 255 : x; }
static inline int sat_s16(int x) { return x < -32768 ? -32768 : x > 32767 ? 32767 : x; }
static inline int subs_u16(int a, int b)      /* _mm_subs_epu16 on values read as uint16 */
{
    const int d = (int)(uint16_t)a - (int)(uint16_t)b;
    return (int16_t)(uint16_t)(d < 0 ? 0 : d);
}
static inline int max_s16(int a, int b) { return (int16_t)a > (int16_t)b ? (int16_t)a : (int16_t)b; }

/* ksw_u8 (size 1) or ksw_i16 (size 2) on profile q */
static orc_kswr_t sw_pass(const prof_t *q, int tlen, const uint8_t *target, int o_del, int e_del, int o_ins,
                          int e_ins, int xtra)
{
    orc_kswr_t r = {0, -1, -1, -1, -1, -1, -1};      /* g_defr, ksw.c:44 */
    const int p = q->p, slen = q->slen, n = slen * p, u8 = q->size == 1;
    const int minsc = (xtra & ORC_KSW_XSUBO) ? xtra & 0xffff : 0x10000;
    const int endsc = (xtra & ORC_KSW_XSTOP) ? xtra & 0xffff : 0x10000;
    const int oe_del = o_del + e_del, oe_ins = o_ins + e_ins;
    int *H0 = calloc(n + 1, sizeof(int)), *H1 = calloc(n + 1, sizeof(int));
    int *E = calloc(n + 1, sizeof(int)), *Hmax = calloc(n + 1, sizeof(int));
    int f[16], h[16], mx[16];
    uint64_t *b = 0;
    int n_b = 0, m_b = 0, gmax = 0, te = -1;
    /* the penalties as the reference broadcasts them: 8 bits (_mm_set1_epi8) or 16 (_mm_set1_epi16) */
    const int pe_del = u8 ? (uint8_t)e_del : (uint16_t)e_del, poe_del = u8 ? (uint8_t)oe_del : (uint16_t)oe_del;
    const int pe_ins = u8 ? (uint8_t)e_ins : (uint16_t)e_ins, poe_ins = u8 ? (uint8_t)oe_ins : (uint16_t)oe_ins;
    for (int i = 0; i < tlen; ++i) {
        const int16_t *S = q->qp + (size_t)target[i] * n;
        for (int l = 0; l < p; ++l) f[l] = 0, mx[l] = 0;
        /* h = H(i-1, -1): the last vector shifted up one lane (ksw.c:141-142) */
        for (int l = p - 1; l > 0; --l) h[l] = slen ? H0[(slen - 1) * p + l - 1] : 0;
        h[0] = 0;
        for (int j = 0; j < slen; ++j) {
            for (int l = 0; l < p; ++l) {
                const int x = j * p + l;
                int hv, e, t;
                if (u8) {
                    hv = sat_u8(sat_u8(h[l] + (uint16_t)S[x]) - q->shift);
                    e = E[x];
                    hv = hv > e ? hv : e;
                    hv = hv > f[l] ? hv : f[l];
                    mx[l] = mx[l] > hv ? mx[l] : hv;
                    H1[x] = hv;
                    e = sat_u8(e - pe_del), t = sat_u8(hv - poe_del);
                    E[x] = e > t ? e : t;
                    f[l] = sat_u8(f[l] - pe_ins), t = sat_u8(hv - poe_ins);
                    f[l] = f[l] > t ? f[l] : t;
                } else {
                    hv = sat_s16(h[l] + S[x]);
                    e = E[x];
                    hv = max_s16(hv, e);
                    hv = max_s16(hv, f[l]);
                    mx[l] = max_s16(mx[l], hv);
                    H1[x] = hv;
                    e = subs_u16(e, pe_del), t = subs_u16(hv, poe_del);
                    E[x] = max_s16(e, t);
                    f[l] = subs_u16(f[l], pe_ins), t = subs_u16(hv, poe_ins);
                    f[l] = max_s16(f[l], t);
                }
                h[l] = H0[x];
            }
        }
#ifndef ORC_SW_LAZY_F_CLOSED_FORM
        /* lazy F (ksw.c:166-177 / 284-295): at most 16 passes, each shifting f up one lane */
        for (int k = 0; k < 16; ++k) {
            for (int l = p - 1; l > 0; --l) f[l] = f[l - 1];
            f[0] = 0;
            int done = 0;
            for (int j = 0; j < slen && !done; ++j) {
                int any = 0;
                for (int l = 0; l < p; ++l) {
                    const int x = j * p + l;
                    int hv;
                    if (u8) {
                        hv = H1[x] > f[l] ? H1[x] : f[l];
                        H1[x] = hv;
                        hv = sat_u8(hv - poe_ins);
                        f[l] = sat_u8(f[l] - pe_ins);
                        any |= sat_u8(f[l] - hv) != 0;
                    } else {
                        hv = max_s16(H1[x], f[l]);
                        H1[x] = hv;
                        hv = subs_u16(hv, poe_ins);
                        f[l] = subs_u16(f[l], pe_ins);
                        any |= (int16_t)f[l] > (int16_t)hv;
                    }
                }
                if (!any) done = 1;
            }
            if (done) break;
        }
#else
        /* Test build only (-DORC_SW_LAZY_F_CLOSED_FORM): the closed form the GPU kernels use
         * where oe_ins >= e_ins as the lanes hold them -- H(l, j) raised to relu(G(l) - j*e_ins),
         * G(0) = 0, G(l) = max(x(l), relu(G(l-1) - slen*e_ins)), x(l) the f leaving lane l-1,
         * applied when a lane fails the reference's first exit test.  The default build runs the
         * loop above, as the reference does. */
        for (int l = p - 1; l > 0; --l) f[l] = f[l - 1];
        f[0] = 0;
        if (slen) {
            int any = 0, h0[16];
            for (int l = 0; l < p; ++l) {
                int hh, fn;
                if (u8) {
                    h0[l] = H1[l] > f[l] ? H1[l] : f[l];
                    hh = sat_u8(h0[l] - poe_ins), fn = sat_u8(f[l] - pe_ins);
                    any |= fn > hh;
                } else {
                    h0[l] = max_s16(H1[l], f[l]);
                    hh = subs_u16(h0[l], poe_ins), fn = subs_u16(f[l], pe_ins);
                    any |= (int16_t)fn > (int16_t)hh;
                }
            }
            if (any) {
                long d = (long)pe_ins * slen, G[16];
                G[0] = f[0];
                for (int l = 1; l < p; ++l) {
                    const long a = G[l - 1] - d > 0 ? G[l - 1] - d : 0;
                    G[l] = f[l] > a ? f[l] : a;
                }
                for (int l = 0; l < p; ++l)
                    for (int j = 0; j < slen; ++j) {
                        const long g = G[l] - (long)pe_ins * j > 0 ? G[l] - (long)pe_ins * j : 0;
                        const int x = j * p + l;
                        if (u8 ? g > H1[x] : g > (int16_t)H1[x]) H1[x] = (int)g;
                    }
            } else {
                for (int l = 0; l < p; ++l) H1[l] = h0[l];
            }
        }
#endif
        int imax = 0;
        for (int l = 0; l < p; ++l) imax = u8 ? (imax > mx[l] ? imax : mx[l]) : max_s16(imax, mx[l]);
        if (!u8) imax = (uint16_t)imax;                 /* _mm_extract_epi16 (ksw.c:249) */
        if (imax >= minsc) {                            /* ksw.c:182-189 */
            if (n_b == 0 || (int32_t)b[n_b - 1] + 1 != i) {
                if (n_b == m_b) m_b = m_b ? m_b << 1 : 8, b = realloc(b, 8 * m_b);
                b[n_b++] = (uint64_t)imax << 32 | (uint32_t)i;
            } else if ((int)(b[n_b - 1] >> 32) < imax) {
                b[n_b - 1] = (uint64_t)imax << 32 | (uint32_t)i;
            }
        }
        if (imax > gmax) {
            gmax = imax, te = i;
            memcpy(Hmax, H1, sizeof(int) * n);
            if ((u8 && gmax + q->shift >= 255) || gmax >= endsc) break;
        }
        int *tmp = H0;
        H0 = H1, H1 = tmp;
    }
    r.score = u8 ? (gmax + q->shift < 255 ? gmax : 255) : gmax;
    r.te = te;
    if (!u8 || r.score != 255) {                        /* qe and the second-best score */
        int best = -1;
        for (int x = 0; x < n; ++x) {
            const int v = u8 ? Hmax[x] : (uint16_t)Hmax[x];
            const int col = x / p + (x % p) * slen;
            if (v > best) best = v, r.qe = col;
            else if (v == best && col < r.qe) r.qe = col;
        }
        if (b) {
            const int d = (r.score + q->max - 1) / q->max;
            const int low = te - d, high = te + d;
            for (int k = 0; k < n_b; ++k) {
                const int e = (int32_t)b[k];
                if ((e < low || e > high) && (int)(b[k] >> 32) > r.score2) r.score2 = b[k] >> 32, r.te2 = e;
            }
        }
    }
    free(b), free(H0), free(H1), free(E), free(Hmax);
    return r;
}

orc_kswr_t orc_ksw_align2(int qlen, const uint8_t *query, int tlen, const uint8_t *target, const int8_t mat[25],
                          int o_del, int e_del, int o_ins, int e_ins, int xtra)
{
    prof_t q;
    qinit(&q, (xtra & ORC_KSW_XBYTE) ? 1 : 2, qlen, query, mat);
    const int size = q.size;
    orc_kswr_t r = sw_pass(&q, tlen, target, o_del, e_del, o_ins, e_ins, xtra);
    free(q.qp);
    if ((xtra & ORC_KSW_XSTART) == 0 || ((xtra & ORC_KSW_XSUBO) && r.score < (xtra & 0xffff))) return r;
    if (r.qe < 0) return r;     /* a saturated byte pass leaves qe at -1; the reference would profile 0 columns */
    /* reversed copies of query[0..qe] and target[0..te], the rest of the target as is (ksw.c:350-354) */
    uint8_t *rq = malloc(r.qe + 1), *rt = malloc(tlen > 0 ? tlen : 1);
    for (int i = 0; i <= r.qe; ++i) rq[i] = query[r.qe - i];
    memcpy(rt, target, tlen);
    for (int i = 0; i <= r.te; ++i) rt[i] = target[r.te - i];
    qinit(&q, size, r.qe + 1, rq, mat);
    const orc_kswr_t rr = sw_pass(&q, tlen, rt, o_del, e_del, o_ins, e_ins, ORC_KSW_XSTOP | r.score);
    free(q.qp), free(rq), free(rt);
    if (r.score == rr.score) r.tb = r.te - rr.te, r.qb = r.qe - rr.qe;
    return r;
}

typedef struct {
    int64_t lo, hi;
    const orc_sw_job_t *jobs;
    const uint8_t *seq;
    const int8_t *mat;
    int o_del, e_del, o_ins, e_ins;
    orc_kswr_t *out;
} sw_range_t;

static void *sw_run(void *arg)
{
    sw_range_t *r = arg;
    for (int64_t i = r->lo; i < r->hi; ++i) {
        const orc_sw_job_t *j = r->jobs + i;
        r->out[i] = orc_ksw_align2(j->qlen, r->seq + j->qoff, j->tlen, r->seq + j->toff, r->mat, r->o_del, r->e_del,
                                   r->o_ins, r->e_ins, j->xtra);
    }
    return 0;
}

void orc_align2_batch(int64_t n, const orc_sw_job_t *jobs, const uint8_t *seq, const int8_t mat[25], int o_del,
                      int e_del, int o_ins, int e_ins, orc_kswr_t *out, int n_threads)
{
    if (n_threads < 1) n_threads = 1;
    if (n_threads > n) n_threads = n > 0 ? (int)n : 1;
    sw_range_t *rs = calloc(n_threads, sizeof(sw_range_t));
    pthread_t *th = calloc(n_threads, sizeof(pthread_t));
    for (int t = 0; t < n_threads; ++t) {
        rs[t] = (sw_range_t){n * t / n_threads, n * (t + 1) / n_threads, jobs, seq, mat, o_del, e_del, o_ins, e_ins, out};
        if (t) pthread_create(&th[t], 0, sw_run, &rs[t]);
    }
    sw_run(&rs[0]);
    for (int t = 1; t < n_threads; ++t) pthread_join(th[t], 0);
    free(rs), free(th);
}
