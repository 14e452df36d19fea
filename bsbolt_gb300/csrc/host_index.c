/*
 * host_index.c -- builds a bisulfite FM-index in BWA's on-disk formats.
 *
 * Produces the files `bwa index -a bwtsw` of BSBolt's BWA fork writes
 * (bsbolt/External/BWA/bwtindex.c:256-321) for a FASTA reference:
 *   .pac   Watson copy with C->T then a Crick copy (<name>_crick_bs) with
 *          G->A (bntseq.c:230-275), 2-bit packed, forward strands only;
 *   .opac  the same two copies unconverted (bwtindex.c:303-304);
 *   .ann / .amb  contig table and N runs (bntseq.c:67-97);
 *   .bwt   BWT of pac + reverse complement (bntseq.c:331-339), $ removed,
 *          128-symbol occurrence blocks interleaved (bwtindex.c:151-173);
 *   .sa    suffix array sampled every 32 rows (bwt.c:61-84, bwt.c:385-407).
 * N bases are replaced by lrand48()&3 after srand48(11), in the same order
 * as the reference, so files match byte for byte.  The suffix array is
 * built with our own SA-IS (Nong, Zhang & Chan 2009); any correct suffix
 * sort gives the same BWT and SA.
 *
 * Host code only: this is how the GPU path's tests and benchmarks get an
 * index where the reference's `bwa index` is not available.
 */
#define _GNU_SOURCE
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ SA-IS */

#define TGET(t, i) ((t)[(i) >> 3] >> ((i) & 7) & 1)
#define TSET(t, i, b) ((b) ? ((t)[(i) >> 3] |= (uint8_t)(1u << ((i) & 7))) : ((t)[(i) >> 3] &= (uint8_t)~(1u << ((i) & 7))))
#define ISLMS(t, i) ((i) > 0 && TGET(t, i) && !TGET(t, (i) - 1))

static void buckets(const int32_t *T, int64_t n, int32_t K, int64_t *bkt, int end)
{
    int64_t i, sum = 0;
    memset(bkt, 0, sizeof(int64_t) * (K + 1));
    for (i = 0; i < n; ++i) ++bkt[T[i]];
    for (i = 0; i <= K; ++i) {
        sum += bkt[i];
        bkt[i] = end ? sum : sum - bkt[i];
    }
}

static void induce(const int32_t *T, int32_t *SA, const uint8_t *t, int64_t n, int32_t K, int64_t *bkt)
{
    int64_t i, j;
    buckets(T, n, K, bkt, 0);
    for (i = 0; i < n; ++i) {
        j = (int64_t)SA[i] - 1;
        if (SA[i] > 0 && !TGET(t, j)) SA[bkt[T[j]]++] = (int32_t)j;
    }
    buckets(T, n, K, bkt, 1);
    for (i = n - 1; i >= 0; --i) {
        j = (int64_t)SA[i] - 1;
        if (SA[i] > 0 && TGET(t, j)) SA[--bkt[T[j]]] = (int32_t)j;
    }
}

/* T[0..n-1] over [0,K) with T[n-1] == 0 the unique smallest symbol. */
static int sais(const int32_t *T, int32_t *SA, int64_t n, int32_t K)
{
    uint8_t *t = (uint8_t *)calloc((size_t)(n >> 3) + 1, 1);
    int64_t *bkt = (int64_t *)malloc(sizeof(int64_t) * ((size_t)K + 1));
    int64_t i, j, n1 = 0;
    int32_t name = 0;
    if (!t || !bkt) { free(t); free(bkt); return -1; }
    TSET(t, n - 1, 1);
    for (i = n - 2; i >= 0; --i)
        TSET(t, i, T[i] < T[i + 1] || (T[i] == T[i + 1] && TGET(t, i + 1)));
    /* stage 1: sort LMS substrings by induction */
    buckets(T, n, K, bkt, 1);
    for (i = 0; i < n; ++i) SA[i] = -1;
    for (i = 1; i < n; ++i)
        if (ISLMS(t, i)) SA[--bkt[T[i]]] = (int32_t)i;
    induce(T, SA, t, n, K, bkt);
    for (i = 0; i < n; ++i)
        if (ISLMS(t, SA[i])) SA[n1++] = SA[i];
    /* name the LMS substrings */
    for (i = n1; i < n; ++i) SA[i] = -1;
    {
        int64_t prev = -1;
        for (i = 0; i < n1; ++i) {
            int64_t pos = SA[i], d;
            int diff = 0;
            for (d = 0; d < n; ++d) {
                if (prev == -1 || T[pos + d] != T[prev + d] || TGET(t, pos + d) != TGET(t, prev + d)) {
                    diff = 1;
                    break;
                } else if (d > 0 && (ISLMS(t, pos + d) || ISLMS(t, prev + d))) {
                    break;
                }
            }
            if (diff) { ++name; prev = pos; }
            SA[n1 + (pos >> 1)] = name - 1;
        }
        for (i = n - 1, j = n - 1; i >= n1; --i)
            if (SA[i] >= 0) SA[j--] = SA[i];
    }
    /* stage 2: sort the reduced string */
    {
        int32_t *s1 = SA + n - n1, *SA1 = SA;
        if (name < n1) {
            if (sais(s1, SA1, n1, name) != 0) { free(t); free(bkt); return -1; }
        } else {
            for (i = 0; i < n1; ++i) SA1[s1[i]] = (int32_t)i;
        }
        /* stage 3: induce the full SA from the sorted LMS suffixes */
        buckets(T, n, K, bkt, 1);
        for (i = 1, j = 0; i < n; ++i)
            if (ISLMS(t, i)) s1[j++] = (int32_t)i;
        for (i = 0; i < n1; ++i) SA1[i] = s1[SA1[i]];
        for (i = n1; i < n; ++i) SA[i] = -1;
        for (i = n1 - 1; i >= 0; --i) {
            j = SA[i];
            SA[i] = -1;
            SA[--bkt[T[j]]] = (int32_t)j;
        }
        induce(T, SA, t, n, K, bkt);
    }
    free(t);
    free(bkt);
    return 0;
}

/* ------------------------------------------------------------- FASTA + pac */

typedef struct {
    char *name, *comment;
    char *seq;
    int64_t len;
} contig_t;

typedef struct {
    int64_t offset;
    int32_t len;
    char amb;
} hole_t;

static const uint8_t *nt4(void)
{
    static uint8_t tab[256];
    static int init = 0;
    if (!init) {
        memset(tab, 4, 256);
        tab['A'] = tab['a'] = 0; tab['C'] = tab['c'] = 1;
        tab['G'] = tab['g'] = 2; tab['T'] = tab['t'] = 3;
        init = 1;
    }
    return tab;
}

static int read_fasta(const char *fn, contig_t **out, int *n_out)
{
    FILE *fp = fopen(fn, "r");
    char *line = NULL;
    size_t cap = 0;
    ssize_t len;
    contig_t *a = NULL;
    int n = 0, m = 0;
    int64_t scap = 0;
    if (!fp) return -1;
    while ((len = getline(&line, &cap, fp)) >= 0) {
        while (len > 0 && (line[len - 1] == '\n' || line[len - 1] == '\r')) line[--len] = 0;
        if (line[0] == '>') {
            char *p = line + 1, *q;
            if (n == m) { m = m ? m * 2 : 16; a = (contig_t *)realloc(a, sizeof(contig_t) * m); }
            q = p;
            while (*q && *q != ' ' && *q != '\t') ++q;
            a[n].name = strndup(p, q - p);
            if (*q) ++q;    /* kseq drops exactly one separator before the comment */
            a[n].comment = *q ? strdup(q) : NULL;
            a[n].seq = NULL; a[n].len = 0; scap = 0;
            ++n;
        } else if (n > 0) {
            contig_t *c = &a[n - 1];
            ssize_t i;
            for (i = 0; i < len; ++i) {
                if (line[i] == ' ' || line[i] == '\t') continue;
                if (c->len == scap) { scap = scap ? scap * 2 : 1 << 16; c->seq = (char *)realloc(c->seq, scap); }
                c->seq[c->len++] = line[i];
            }
        }
    }
    free(line);
    fclose(fp);
    *out = a;
    *n_out = n;
    return 0;
}

#define SETPAC(pac, l, c) ((pac)[(l) >> 2] |= (uint8_t)((c) << ((~(l) & 3) << 1)))
#define GETPAC(pac, l) ((pac)[(l) >> 2] >> ((~(l) & 3) << 1) & 3)

/* Pack Watson then Crick copies (bntseq.c:230-275); conversion 1 = bisulfite. */
static uint8_t *pack(const contig_t *c, int n, int conversion, int64_t *l_pac,
                     hole_t **holes, int *n_holes, int32_t *n_ambs)
{
    const uint8_t *tab = nt4();
    int64_t total = 0, l = 0;
    int k, pass, nh = 0, mh = 0;
    uint8_t *pac;
    hole_t *h = NULL;
    for (k = 0; k < n; ++k) total += c[k].len;
    pac = (uint8_t *)calloc((size_t)(2 * total) / 4 + 2, 1);
    srand48(11);
    for (pass = 0; pass < 2; ++pass) {
        for (k = 0; k < n; ++k) {
            int64_t i;
            int lasts = 0;
            int32_t na = 0;
            for (i = 0; i < c[k].len; ++i) {
                int ch = (unsigned char)c[k].seq[i];
                int b = tab[ch];
                if (conversion) {
                    if (pass == 1) { if (b == 2) b = 0; }
                    else { if (b == 1) b = 3; }
                }
                if (b >= 4) {
                    if (lasts == ch) {
                        ++h[nh - 1].len;
                    } else {
                        if (nh == mh) { mh = mh ? mh * 2 : 16; h = (hole_t *)realloc(h, sizeof(hole_t) * mh); }
                        h[nh].offset = l;
                        h[nh].len = 1;
                        h[nh].amb = (char)ch;
                        ++nh;
                        ++na;
                    }
                }
                lasts = ch;
                if (b >= 4) b = (int)(lrand48() & 3);
                SETPAC(pac, l, b);
                ++l;
            }
            n_ambs[pass * n + k] = na;
        }
    }
    *l_pac = l;
    *holes = h;
    *n_holes = nh;
    return pac;
}

static int write_pac(const char *fn, const uint8_t *pac, int64_t l_pac)
{
    FILE *fp = fopen(fn, "wb");
    uint8_t ct;
    if (!fp) return -1;
    fwrite(pac, 1, (size_t)(l_pac >> 2) + ((l_pac & 3) == 0 ? 0 : 1), fp);
    if (l_pac % 4 == 0) { ct = 0; fwrite(&ct, 1, 1, fp); }
    ct = (uint8_t)(l_pac % 4);
    fwrite(&ct, 1, 1, fp);
    return fclose(fp);
}

static int write_ann_amb(const char *prefix, const contig_t *c, int n, int64_t l_pac,
                         const hole_t *h, int nh, const int32_t *n_ambs)
{
    char fn[4096];
    FILE *fp;
    int pass, k;
    int64_t off = 0;
    snprintf(fn, sizeof fn, "%s.ann", prefix);
    if (!(fp = fopen(fn, "w"))) return -1;
    fprintf(fp, "%lld %d %u\n", (long long)l_pac, 2 * n, 11u);
    for (pass = 0; pass < 2; ++pass) {
        for (k = 0; k < n; ++k) {
            const char *anno = c[k].comment ? c[k].comment : "(null)";
            if (pass == 0) fprintf(fp, "%d %s", 0, c[k].name);
            else fprintf(fp, "%d %s_crick_bs", 0, c[k].name);
            if (anno[0]) fprintf(fp, " %s\n", anno);
            else fprintf(fp, "\n");
            fprintf(fp, "%lld %d %d\n", (long long)off, (int)c[k].len, n_ambs[pass * n + k]);
            off += c[k].len;
        }
    }
    fclose(fp);
    snprintf(fn, sizeof fn, "%s.amb", prefix);
    if (!(fp = fopen(fn, "w"))) return -1;
    fprintf(fp, "%lld %d %u\n", (long long)l_pac, 2 * n, (unsigned)nh);
    for (k = 0; k < nh; ++k) fprintf(fp, "%lld %d %c\n", (long long)h[k].offset, h[k].len, h[k].amb);
    return fclose(fp);
}

/* --------------------------------------------------------- BWT + SA files */

/* base at position p of the text bwa index sorts: the pac, then its reverse complement */
static inline int text_at(const uint8_t *pac, int64_t l_pac, int64_t p)
{
    return p < l_pac ? GETPAC(pac, p) : 3 - GETPAC(pac, 2 * l_pac - 1 - p);
}

/* .bwt and .sa from the suffix array of the text + '$' (n + 1 rows, in sa32 or sa64) */
static int write_bwt_sa_from(const char *prefix, const uint8_t *pac, int64_t l_pac, int sa_intv, const int32_t *sa32,
                             const int64_t *sa64)
{
    const int64_t n = 2 * l_pac;
    uint64_t L2[5] = {0, 0, 0, 0, 0}, primary = 0, cnt[4] = {0, 0, 0, 0};
    int64_t i, k, r, n_occ, bwt_words, n_sa;
    uint32_t *buf;
    char fn[4096];
    FILE *fp;
    for (i = 0; i < n; ++i) ++L2[text_at(pac, l_pac, i) + 1];
    for (i = 2; i <= 4; ++i) L2[i] += L2[i - 1];
    /* interleaved BWT: 4 x u64 counts then 8 words per 128 symbols, plus a final count block */
    n_occ = (n + 127) / 128 + 1;
    bwt_words = (n + 15) / 16 + n_occ * 8;
    buf = (uint32_t *)calloc((size_t)bwt_words, 4);
    if (!buf) return -3;
    for (r = 0, i = 0, k = 0; r <= n; ++r) {
        const int64_t s = sa32 ? (int64_t)sa32[r] : sa64[r];
        int c;
        if (s == 0) { primary = (uint64_t)r; continue; }
        c = text_at(pac, l_pac, s - 1);
        if (i % 128 == 0) { memcpy(buf + k, cnt, 32); k += 8; }
        if (i % 16 == 0) ++k;
        buf[k - 1] |= (uint32_t)c << ((15 - (i & 15)) << 1);
        ++cnt[c];
        ++i;
    }
    memcpy(buf + k, cnt, 32);
    k += 8;
    snprintf(fn, sizeof fn, "%s.bwt", prefix);
    if (!(fp = fopen(fn, "wb"))) { free(buf); return -1; }
    fwrite(&primary, 8, 1, fp);
    fwrite(L2 + 1, 8, 4, fp);
    fwrite(buf, 4, (size_t)k, fp);
    fclose(fp);
    free(buf);

    /* sampled suffix array: sa[r/intv] = SA[r] for r % intv == 0, sa[0] = -1 (not stored) */
    n_sa = (n + sa_intv) / sa_intv;
    snprintf(fn, sizeof fn, "%s.sa", prefix);
    if (!(fp = fopen(fn, "wb"))) return -1;
    {
        uint64_t v = (uint64_t)sa_intv, sl = (uint64_t)n;
        fwrite(&primary, 8, 1, fp);
        fwrite(L2 + 1, 8, 4, fp);
        fwrite(&v, 8, 1, fp);
        fwrite(&sl, 8, 1, fp);
        for (i = 1; i < n_sa; ++i) {
            uint64_t x = (uint64_t)(sa32 ? (int64_t)sa32[i * sa_intv] : sa64[i * sa_intv]);
            fwrite(&x, 8, 1, fp);
        }
    }
    return fclose(fp);
}

static int write_bwt_sa(const char *prefix, const uint8_t *pac, int64_t l_pac, int sa_intv)
{
    const int64_t n = 2 * l_pac;                /* text length without the sentinel */
    int32_t *T, *SA;
    int64_t i;
    int rc;
    if (n + 1 > 0x7fffffffLL) return -2;       /* int32 SA-IS limit */
    T = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 1));
    SA = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 1));
    if (!T || !SA) { free(T); free(SA); return -3; }
    for (i = 0; i < n; ++i) T[i] = text_at(pac, l_pac, i) + 1;
    T[n] = 0;
    if (sais(T, SA, n + 1, 5) != 0) { free(T); free(SA); return -3; }
    free(T);
    rc = write_bwt_sa_from(prefix, pac, l_pac, sa_intv, SA, NULL);
    free(SA);
    return rc;
}

/* .bwt and .sa of <prefix> from a suffix array sorted elsewhere (the GPU's), 2*l_pac + 1 rows
 * of int64, and the converted pac of <prefix>.pac. */
int bsbh_write_bwt_sa64(const char *prefix, const uint8_t *pac, int64_t l_pac, const int64_t *sa, int sa_intv)
{
    if (!prefix || !pac || !sa || l_pac < 1 || sa_intv < 1) return -1;
    return write_bwt_sa_from(prefix, pac, l_pac, sa_intv, NULL, sa);
}

/* .bwt and .sa of <prefix> from a BWT and sampled suffix array built elsewhere (the GPU's
 * bsb_build_bwt): n = 2*l_pac symbols, bwt packed 16 to a word (first symbol in the top bits,
 * the row of suffix 0 left out), primary = that row, sa[k] = SA[k * sa_intv] for k < n_sa =
 * (n + sa_intv) / sa_intv.  The symbol counts L2 are the BWT's own (it permutes the text). */
int bsbh_write_bwt_packed(const char *prefix, int64_t n, const uint32_t *bwt, uint64_t primary, const uint64_t *sa,
                          int sa_intv)
{
    uint64_t L2[5] = {0, 0, 0, 0, 0}, cnt[4] = {0, 0, 0, 0};
    const int64_t n_words = (n + 15) / 16, n_occ = (n + 127) / 128 + 1, n_sa = (n + sa_intv) / sa_intv;
    int64_t w, k = 0, i;
    uint32_t *buf;
    char fn[4096];
    FILE *fp;
    if (!prefix || !bwt || !sa || n < 1 || sa_intv < 1 || primary > (uint64_t)n) return -1;
    uint32_t by4[256];           /* the symbol counts of a byte (4 symbols), one per byte lane */
    buf = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(n_words + n_occ * 8));
    if (!buf) return -3;
    for (i = 0; i < 256; ++i) {
        int j;
        by4[i] = 0;
        for (j = 0; j < 4; ++j) by4[i] += 1u << ((i >> (j << 1) & 3) << 3);
    }
    /* interleaved: the counts before every 128 symbols (4 x u64), then their 8 words */
    for (w = 0; w < n_words; ++w) {
        const uint32_t x = bwt[w];
        const int valid = (int)(n - w * 16 < 16 ? n - w * 16 : 16);
        int j;
        if (w % 8 == 0) { memcpy(buf + k, cnt, 32); k += 8; }
        buf[k++] = x;
        if (valid == 16) {       /* at most 16 of a symbol: the byte lanes do not carry */
            const uint32_t c = by4[x & 255] + by4[x >> 8 & 255] + by4[x >> 16 & 255] + by4[x >> 24];
            for (j = 0; j < 4; ++j) cnt[j] += c >> (j << 3) & 255;
        } else {
            for (j = 0; j < valid; ++j) ++cnt[x >> ((15 - j) << 1) & 3];
        }
    }
    memcpy(buf + k, cnt, 32);
    k += 8;
    for (i = 0; i < 4; ++i) L2[i + 1] = L2[i] + cnt[i];
    snprintf(fn, sizeof fn, "%s.bwt", prefix);
    if (!(fp = fopen(fn, "wb"))) { free(buf); return -1; }
    fwrite(&primary, 8, 1, fp);
    fwrite(L2 + 1, 8, 4, fp);
    if (fwrite(buf, 4, (size_t)k, fp) != (size_t)k) { fclose(fp); free(buf); return -1; }
    free(buf);
    if (fclose(fp)) return -1;
    snprintf(fn, sizeof fn, "%s.sa", prefix);
    if (!(fp = fopen(fn, "wb"))) return -1;
    {
        const uint64_t v = (uint64_t)sa_intv, sl = (uint64_t)n;
        fwrite(&primary, 8, 1, fp);
        fwrite(L2 + 1, 8, 4, fp);
        fwrite(&v, 8, 1, fp);
        fwrite(&sl, 8, 1, fp);
        if (n_sa > 1 && fwrite(sa + 1, 8, (size_t)(n_sa - 1), fp) != (size_t)(n_sa - 1)) { fclose(fp); return -1; }
    }
    return fclose(fp);
}

static int index_fasta(const char *fasta, const char *prefix, int with_bwt, int64_t *l_pac_out);

/* Build <prefix>.{pac,opac,ann,amb,bwt,sa} from a FASTA file.  Returns 0 or a negative code. */
int bsbh_index_fasta(const char *fasta, const char *prefix)
{
    return index_fasta(fasta, prefix, 1, NULL);
}

/* The same without .bwt / .sa (their suffix array is sorted elsewhere); *l_pac receives the
 * length of the converted pac. */
int bsbh_index_fasta_nobwt(const char *fasta, const char *prefix, int64_t *l_pac)
{
    return index_fasta(fasta, prefix, 0, l_pac);
}

static int index_fasta(const char *fasta, const char *prefix, int with_bwt, int64_t *l_pac_out)
{
    contig_t *c = NULL;
    int n = 0, nh = 0, nh2 = 0, k, rc;
    int64_t l_pac = 0, l2;
    hole_t *h = NULL, *h2 = NULL;
    int32_t *na, *na2;
    uint8_t *pac, *opac;
    char fn[4096];
    if (read_fasta(fasta, &c, &n) != 0 || n == 0) return -1;
    na = (int32_t *)calloc(2 * n, sizeof(int32_t));
    na2 = (int32_t *)calloc(2 * n, sizeof(int32_t));
    pac = pack(c, n, 1, &l_pac, &h, &nh, na);
    opac = pack(c, n, 0, &l2, &h2, &nh2, na2);
    snprintf(fn, sizeof fn, "%s.pac", prefix);
    rc = write_pac(fn, pac, l_pac);
    snprintf(fn, sizeof fn, "%s.opac", prefix);
    if (!rc) rc = write_pac(fn, opac, l2);
    if (!rc) rc = write_ann_amb(prefix, c, n, l_pac, h, nh, na);
    if (!rc && with_bwt) rc = write_bwt_sa(prefix, pac, l_pac, 32);
    if (l_pac_out) *l_pac_out = l_pac;
    for (k = 0; k < n; ++k) { free(c[k].name); free(c[k].comment); free(c[k].seq); }
    free(c); free(h); free(h2); free(na); free(na2); free(pac); free(opac);
    return rc;
}

/* Suffix array of an nt4 text (values 0..3) for tests: SA of text+'$' (n+1 entries). */
int bsbh_suffix_array(const uint8_t *text, int64_t n, int32_t *sa_out)
{
    int32_t *T = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 1));
    int64_t i;
    int rc;
    if (!T) return -3;
    for (i = 0; i < n; ++i) T[i] = text[i] + 1;
    T[n] = 0;
    rc = sais(T, sa_out, n + 1, 5);
    free(T);
    return rc;
}
