/*
 * bseq_fast.c -- bseq_read (bsbolt/External/BWA/bwa.c:73-143) for plain four-line FASTQ, with
 * the per-read copies and conversions on threads.
 *
 * BWA's input step parses one record at a time with kseq (kseq.h:175-215) and converts every
 * read (kseq2bseq1, bwa.c:44-71) on the pipeline's input thread; with the alignment on the GPU
 * that thread sets the pace of `bwa mem`.  bseq_read_fast returns the same bseq1_t array.  It
 * takes the stream's bytes over from the kstream, finds the batch's records with a line scan
 * (the sequential part: memchr), checks that kseq would read each record the same way, and
 * builds the entries on threads.  A record it does not take -- FASTA, a sequence or quality
 * over several lines, CR or NUL bytes, an empty sequence line, bytes before a header, a last
 * record without its newline -- hands the unread bytes back to the kstream and calls the
 * reference's own bseq_read, for that batch and every later one.  BSB_FASTQ_READER=0 keeps
 * the reference's reader throughout.  With the native output step (sam_out.c) a batch's names,
 * bases, qualities and original bases are one allocation, which that step frees at once.
 *
 * Link with -Wl,--wrap=bseq_read and call bseq_read_fast from __wrap_bseq_read.
 */
#include <ctype.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>
#include <zlib.h>

#include "bntseq.h"
#include "bs_helpers.h"
#include "bwa.h"
#include "kseq.h"
KSEQ_DECLARE(gzFile)

#include "bwamem_gpu.h"

bseq1_t *__real_bseq_read(int64_t chunk_size, int *n_, void *ks1_, void *ks2_, int64_t *s, int conversion,
                          int undirectional, float substitution_proportion);

/* ---- the bytes of one input stream ---------------------------------------- */

typedef struct {
    const kseq_t *ks;     /* the kseq this state serves */
    char *buf;            /* bytes taken from the kstream and the file; [beg, end) not yet read */
    size_t beg, end, cap;
    int eof;              /* the file has no more bytes */
    int off;              /* the reference's reader owns the stream from now on */
} fq_stream_t;

static fq_stream_t g_fq[2];

static fq_stream_t *fq_find(const kseq_t *ks)
{
    int i;
    for (i = 0; i < 2; ++i)
        if (g_fq[i].ks == ks) return &g_fq[i];
    return 0;
}

/* Takes the stream over from kseq (its buffered bytes come first); 0 without a free slot. */
static fq_stream_t *fq_take(kseq_t *ks)
{
    int i;
    for (i = 0; i < 2; ++i)
        if (!g_fq[i].ks) {
            kstream_t *f = ks->f;
            fq_stream_t *st = &g_fq[i];
            memset(st, 0, sizeof *st);
            st->ks = ks;
            st->cap = 1 << 24;
            st->buf = (char *)malloc(st->cap);
            if (!st->buf) return 0;
            /* what kseq has buffered comes first */
            if (f->end > f->begin) {
                memcpy(st->buf, f->buf + f->begin, (size_t)(f->end - f->begin));
                st->end = (size_t)(f->end - f->begin);
            }
            f->begin = f->end;
            st->eof = f->is_eof;
            return st;
        }
    return 0;                      /* more than two streams: not the `bwa mem` input */
}

/* The unread bytes to the front of the buffer (between batches: no record offsets are held). */
static void fq_compact(fq_stream_t *st)
{
    if (st->beg > 0) {
        memmove(st->buf, st->buf + st->beg, st->end - st->beg);
        st->end -= st->beg;
        st->beg = 0;
    }
}

/* At least `want` unread bytes, or every byte left in the file.  0 on success, -1 on a read
 * error or no memory (the caller hands over to the reference's reader). */
static int fq_fill(fq_stream_t *st, size_t want)
{
    while (!st->eof && st->end - st->beg < want) {
        const size_t chunk = 1 << 22;
        int r;
        if (st->end + chunk > st->cap) {
            char *nb;
            size_t nc = st->cap * 2;
            while (st->end + chunk > nc) nc *= 2;
            if (!(nb = (char *)realloc(st->buf, nc))) return -1;
            st->buf = nb, st->cap = nc;
        }
        r = gzread(st->ks->f->f, st->buf + st->end, (unsigned)chunk);
        if (r < 0) return -1;
        if (r == 0) st->eof = 1;
        st->end += (size_t)r;
    }
    return 0;
}

/* The position of the next '\n' at or after p, reading more of the file as needed; -1 when the
 * file ends first (or on a read error). */
static int64_t fq_line_end(fq_stream_t *st, size_t p)
{
    for (;;) {
        const char *q = p < st->end ? (const char *)memchr(st->buf + p, '\n', st->end - p) : 0;
        size_t have;
        if (q) return q - st->buf;
        if (st->eof) return -1;
        have = st->end - st->beg;
        if (fq_fill(st, have + (1 << 20)) < 0) return -1;
    }
}

/* Back to kseq: the unread bytes become the kstream's buffer (at least its 16 kB, which kseq
 * refills in place), every later batch goes to the reference's reader. */
static void fq_hand_back(fq_stream_t *st)
{
    kstream_t *f;
    size_t left, sz;
    unsigned char *nb;
    if (!st || st->off) return;
    f = st->ks->f;
    left = st->end - st->beg;
    sz = left > 16384 ? left : 16384;
    nb = (unsigned char *)malloc(sz);
    if (nb) {
        memcpy(nb, st->buf + st->beg, left);
        free(f->buf);
        f->buf = nb, f->begin = 0, f->end = (int)left;
        f->is_eof = st->eof;
    }
    free(st->buf);
    st->buf = 0, st->beg = st->end = st->cap = 0;
    st->off = 1;
}

/* ---- records -------------------------------------------------------------- */

typedef struct {
    int64_t name, cmt, seq, qual;  /* offsets into the stream's buffer; cmt < 0: no comment */
    int name_l, cmt_l, seq_l;      /* the quality has seq_l bytes */
} fq_rec_t;

/* kseq_read (kseq.h:175-215) of one four-line record at st->beg, as it would read it:
 * 1 = a record (st->beg moves past it), 0 = no bytes left, -1 = not a record taken here. */
static int fq_record(fq_stream_t *st, fq_rec_t *r)
{
    const size_t p = st->beg;
    int64_t e1, e2, e3, e4, k;
    const char *b;
    if (fq_fill(st, 1) < 0) return -1;
    if (p >= st->end) return st->eof ? 0 : -1;
    if ((e1 = fq_line_end(st, p)) < 0 || (e2 = fq_line_end(st, (size_t)e1 + 1)) < 0 ||
        (e3 = fq_line_end(st, (size_t)e2 + 1)) < 0 || (e4 = fq_line_end(st, (size_t)e3 + 1)) < 0)
        return -1;
    b = st->buf;                                      /* after the reads: the buffer may have moved */
    if (b[p] != '@') return -1;                       /* kseq would skip to the next '@' or '>' */
    if (memchr(b + p, '\r', (size_t)(e4 - (int64_t)p)) || memchr(b + p, 0, (size_t)(e4 - (int64_t)p)))
        return -1;
    /* header: the name up to the first white space, the comment after it (kseq.h:186-187) */
    for (k = (int64_t)p + 1; k < e1 && !isspace((unsigned char)b[k]); ++k) {}
    r->name = (int64_t)p + 1, r->name_l = (int)(k - ((int64_t)p + 1));
    if (k < e1) r->cmt = k + 1, r->cmt_l = (int)(e1 - (k + 1));
    else r->cmt = -1, r->cmt_l = 0;
    /* one sequence line, then the '+' line (kseq.h:192-209) */
    if (e2 == e1 + 1) return -1;                      /* an empty line: kseq skips it */
    if (b[e1 + 1] == '>' || b[e1 + 1] == '+' || b[e1 + 1] == '@') return -1;
    if (b[e2 + 1] != '+') return -1;                  /* the sequence goes on over more lines */
    r->seq = e1 + 1, r->seq_l = (int)(e2 - (e1 + 1));
    /* one quality line of the sequence's length (kseq.h:211-213) */
    if (e4 - (e3 + 1) != r->seq_l) return -1;
    r->qual = e3 + 1;
    st->beg = (size_t)e4 + 1;
    return 1;
}

/* trim_readno (bwa.c:27-31) on a name of length *l */
static void fq_trim(const char *name, int *l)
{
    if (*l > 2 && name[*l - 2] == '/' && isdigit((unsigned char)name[*l - 1])) *l -= 2;
}

static char *fq_dup(const char *s, int l)
{
    char *d = (char *)malloc((size_t)l + 1);
    memcpy(d, s, (size_t)l);
    d[l] = 0;
    return d;
}

/* One entry of the batch: which stream, which record, the name length after trimming, and
 * kseq2bseq1's first / read_group / substitution_pattern. */
typedef struct {
    int stream, rec, name_l;
    int first, read_group, pattern;
} fq_entry_t;

typedef struct {
    fq_stream_t *st[2];
    const fq_rec_t *rec[2];
    const fq_entry_t *ent;
    bseq1_t *seqs;
    int conversion;
    int64_t next, n;
} fq_build_t;

/* The strings of entry i, allocated on the calling thread: BWA frees them in its output step
 * (bs_sorter.cpp:152-156) on the pipeline thread that read the batch, and a free into another
 * thread's heap arena takes that arena's lock, against the worker threads allocating there. */
static void fq_alloc1(fq_build_t *B, int64_t i)
{
    const fq_entry_t *e = &B->ent[i];
    const fq_rec_t *r = &B->rec[e->stream][e->rec];
    bseq1_t *s = &B->seqs[i];
    memset(s, 0, sizeof *s);
    s->name = (char *)malloc((size_t)e->name_l + 1);
    s->comment = r->cmt_l ? (char *)malloc((size_t)r->cmt_l + 1) : 0;
    s->seq = (char *)malloc((size_t)r->seq_l + 1);
    s->qual = r->seq_l ? (char *)malloc((size_t)r->seq_l + 1) : 0;
    s->oseq = B->conversion ? (char *)malloc((size_t)r->seq_l + 1) : 0;
}

/* With the native output step (sam_out.c), the batch's names, bases, qualities and original
 * bases are carved from one block, the first read's name at its start, which the output step
 * frees at once (sam_out_take_block); comments stay separate, since mem's input step frees
 * them itself unless -C (fastmap.c:26-30).  0 when the block cannot be had. */
static int fq_alloc_block(fq_build_t *B)
{
    size_t total = 0;
    int64_t i;
    char *p;
    for (i = 0; i < B->n; ++i) {
        const fq_entry_t *e = &B->ent[i];
        const int l = B->rec[e->stream][e->rec].seq_l;
        total += (size_t)e->name_l + 1 + (size_t)l + 1 + (l ? (size_t)l + 1 : 0) + (B->conversion ? (size_t)l + 1 : 0);
    }
    if (B->n == 0 || !(p = (char *)malloc(total))) return 0;
    for (i = 0; i < B->n; ++i) {
        const fq_entry_t *e = &B->ent[i];
        const fq_rec_t *r = &B->rec[e->stream][e->rec];
        bseq1_t *s = &B->seqs[i];
        memset(s, 0, sizeof *s);
        s->name = p, p += e->name_l + 1;
        s->seq = p, p += r->seq_l + 1;
        if (r->seq_l) s->qual = p, p += r->seq_l + 1;
        if (B->conversion) s->oseq = p, p += r->seq_l + 1;
        s->comment = r->cmt_l ? (char *)malloc((size_t)r->cmt_l + 1) : 0;
    }
    sam_out_give_block(B->seqs[0].name);
    return 1;
}

static void fq_copy(char *d, const char *src, int l)
{
    memcpy(d, src, (size_t)l);
    d[l] = 0;
}

/* kseq2bseq1 (bwa.c:44-71) of entry i, into the strings fq_alloc1 made */
static void fq_build1(fq_build_t *B, int64_t i)
{
    const fq_entry_t *e = &B->ent[i];
    const fq_rec_t *r = &B->rec[e->stream][e->rec];
    const char *b = B->st[e->stream]->buf;
    bseq1_t *s = &B->seqs[i];
    int k;
    fq_copy(s->name, b + r->name, e->name_l);
    if (s->comment) fq_copy(s->comment, b + r->cmt, r->cmt_l);
    fq_copy(s->seq, b + r->seq, r->seq_l);
    if (s->qual) fq_copy(s->qual, b + r->qual, r->seq_l);
    s->l_seq = r->seq_l;
    s->first = e->first;
    s->read_group = e->read_group;
    s->subsitution_pattern = e->pattern;
    s->conversion = B->conversion;
    s->id = (int)i;
    if (B->conversion) {
        fq_copy(s->oseq, b + r->seq, r->seq_l);
        bsConversion(s->seq, s->subsitution_pattern, s->l_seq);
        for (k = 0; k < s->l_seq; ++k) s->oseq[k] = s->oseq[k] < 4 ? s->oseq[k] : nst_nt4_table[(int)s->oseq[k]];
    }
}

static void *fq_worker(void *arg)
{
    fq_build_t *B = (fq_build_t *)arg;
    for (;;) {
        const int64_t a = __atomic_fetch_add(&B->next, 1024, __ATOMIC_RELAXED);
        int64_t i;
        if (a >= B->n) break;
        for (i = a; i < B->n && i < a + 1024; ++i) fq_build1(B, i);
    }
    return 0;
}

static void fq_build_all(fq_build_t *B)
{
    pthread_t th[32];
    long nc = sysconf(_SC_NPROCESSORS_ONLN);
    int t, nt = nc < 1 ? 1 : nc > 32 ? 32 : (int)nc, started = 0;
    if (nt > (B->n + 1023) / 1024) nt = (int)((B->n + 1023) / 1024);
    for (t = 1; t < nt; ++t) {
        if (pthread_create(&th[t], 0, fq_worker, B)) break;
        started = t;
    }
    fq_worker(B);
    for (t = 1; t <= started; ++t) pthread_join(th[t], 0);
}

/* ---- bseq_read ------------------------------------------------------------ */

typedef struct {
    fq_rec_t *a;
    int n, m;
} fq_recv_t;

static int fq_push(fq_recv_t *v, const fq_rec_t *r)
{
    if (v->n == v->m) {
        int m = v->m ? v->m * 2 : 4096;
        fq_rec_t *a = (fq_rec_t *)realloc(v->a, sizeof(fq_rec_t) * m);
        if (!a) return -1;
        v->a = a, v->m = m;
    }
    v->a[v->n++] = *r;
    return 0;
}

static int fq_push_entry(fq_entry_t **ent, int64_t *n, int64_t *m, const fq_entry_t *e)
{
    if (*n == *m) {
        int64_t nm = *m ? *m * 2 : 4096;
        fq_entry_t *a = (fq_entry_t *)realloc(*ent, sizeof(fq_entry_t) * nm);
        if (!a) return -1;
        *ent = a, *m = nm;
    }
    (*ent)[(*n)++] = *e;
    return 0;
}

/* assessConversion (bs_helpers.cpp:41-62) on the records' sequences (NUL-terminated copies) */
static int fq_assess(fq_stream_t *s1, const fq_rec_t *r1, fq_stream_t *s2, const fq_rec_t *r2, float prop)
{
    char *a = fq_dup(s1->buf + r1->seq, r1->seq_l), *b = r2 ? fq_dup(s2->buf + r2->seq, r2->seq_l) : a;
    const int t = assessConversion(a, b, r2 != 0, prop);
    if (b != a) free(b);
    free(a);
    return t;
}

bseq1_t *bseq_read_fast(int64_t chunk_size, int *n_, void *ks1_, void *ks2_, int64_t *s, int conversion,
                        int undirectional, float substitution_proportion)
{
    static int enabled = -1;
    kseq_t *ks = (kseq_t *)ks1_, *ks2 = (kseq_t *)ks2_;
    fq_stream_t *st1, *st2 = 0;
    size_t beg1, beg2 = 0;
    fq_recv_t v1 = {0, 0, 0}, v2 = {0, 0, 0};
    fq_entry_t *ent = 0;
    int64_t n = 0, m_ent = 0, size = 0;
    bseq1_t *seqs;
    fq_build_t B;
    if (enabled < 0) {
        const char *e = getenv("BSB_FASTQ_READER");
        enabled = !(e && e[0] == '0');
    }
    if (!enabled) return __real_bseq_read(chunk_size, n_, ks1_, ks2_, s, conversion, undirectional,
                                          substitution_proportion);
    st1 = fq_find(ks);
    st2 = ks2 ? fq_find(ks2) : 0;
    /* kseq keeps last_char 0 between FASTQ records; a header char it has already read (FASTA) or
     * a stream handed back stays with the reference's reader */
    if ((st1 && st1->off) || (st2 && st2->off) || ks->last_char || (ks2 && ks2->last_char)) goto reference;
    if (!st1 && !(st1 = fq_take(ks))) goto reference;
    if (ks2 && !st2 && !(st2 = fq_take(ks2))) goto reference;
    fq_compact(st1);
    if (st2) fq_compact(st2);
    beg1 = st1->beg;
    if (st2) beg2 = st2->beg;
    for (;;) {
        fq_rec_t r1, r2;
        fq_entry_t e;
        int pattern = 0, compare = 0, k, l1, l2 = 0;
        k = fq_record(st1, &r1);
        if (k < 0) goto undo;
        if (k == 0) {               /* the first file is done */
            if (n == 0) goto undo;  /* the reference's reader gives the end (and its warning) */
            break;
        }
        if (st2) {
            k = fq_record(st2, &r2);
            if (k <= 0) goto undo;  /* the reference's reader has the warning of a shorter 2nd file */
        }
        if (undirectional) {        /* bwa.c:93-101 */
            const int t = fq_assess(st1, &r1, st2, st2 ? &r2 : 0, substitution_proportion);
            if (t == 2) compare = 1;
            else pattern = t;
            if (pattern > 1) fprintf(stderr, "conversion error\n");
        }
        if (fq_push(&v1, &r1) < 0 || (st2 && fq_push(&v2, &r2) < 0)) goto undo;
        l1 = r1.name_l;
        fq_trim(st1->buf + r1.name, &l1);
        e.stream = 0, e.rec = v1.n - 1, e.name_l = l1, e.first = 0, e.read_group = 0, e.pattern = pattern;
        if (fq_push_entry(&ent, &n, &m_ent, &e) < 0) goto undo;
        size += r1.seq_l;
        if (st2) {
            l2 = r2.name_l;
            fq_trim(st2->buf + r2.name, &l2);
            e.stream = 1, e.rec = v2.n - 1, e.name_l = l2, e.first = 1, e.read_group = 0, e.pattern = pattern ? 0 : 1;
            if (fq_push_entry(&ent, &n, &m_ent, &e) < 0) goto undo;
            size += r2.seq_l;
        }
        if (compare) {              /* the read (pair) again with the other pattern; the names trimmed again */
            fq_trim(st1->buf + r1.name, &l1);
            e.stream = 0, e.rec = v1.n - 1, e.name_l = l1, e.first = 0, e.read_group = 1, e.pattern = 1;
            if (fq_push_entry(&ent, &n, &m_ent, &e) < 0) goto undo;
            size += r1.seq_l;
            if (st2) {
                fq_trim(st2->buf + r2.name, &l2);
                e.stream = 1, e.rec = v2.n - 1, e.name_l = l2, e.first = 1, e.read_group = 1, e.pattern = 0;
                if (fq_push_entry(&ent, &n, &m_ent, &e) < 0) goto undo;
                size += r2.seq_l;
            }
        }
        if (size >= chunk_size && (n & 1) == 0) break;
    }
    seqs = (bseq1_t *)malloc(sizeof(bseq1_t) * (n + 2));
    if (!seqs) goto undo;
    B.st[0] = st1, B.st[1] = st2, B.rec[0] = v1.a, B.rec[1] = v2.a, B.ent = ent, B.seqs = seqs;
    B.conversion = conversion, B.next = 0, B.n = n;
    if (!sam_out_enabled() || !fq_alloc_block(&B)) {
        int64_t i;
        for (i = 0; i < n; ++i) fq_alloc1(&B, i);
    }
    fq_build_all(&B);
    free(v1.a); free(v2.a); free(ent);
    *n_ = (int)n;
    return seqs;

undo:                               /* nothing of this batch is taken: the bytes go back to kseq */
    st1->beg = beg1;
    if (st2) st2->beg = beg2;
    free(v1.a); free(v2.a); free(ent);
reference:
    fq_hand_back(st1);
    fq_hand_back(st2);
    return __real_bseq_read(chunk_size, n_, ks1_, ks2_, s, conversion, undirectional, substitution_proportion);
}
