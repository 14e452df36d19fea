/*
 * sam_out.c -- the output step of BSBolt's `bwa mem` (fastmap.c:60-71 with samSorter,
 * bsbolt/External/BWA/bs_sorter.cpp), with the same bytes on stdout and the same BSStat
 * lines on stderr, the copying done on threads and one write per batch.
 *
 * The reference's step takes the batch's reads in order (the first, then every read with a
 * SAM record), groups consecutive reads of one name into two queues by read_group, and at
 * each change of name (and at the end) writes one queue: the one with the higher summed
 * alignment score, or on a tie the first queue with every read rewritten as unmapped and
 * counted as bisulfite-ambiguous (setUnmapped, bs_sorter.cpp:51-82).  Each written read is
 * counted by its mapping class; the other queue is dropped.  Here the same decisions are made
 * in one pass over the reads (it is sequential, and cheap), then the records are measured and
 * copied into one buffer on threads, each record freed by the thread that copied it (worker2's
 * threads allocated them), the buffer written with one fwrite, and the reads' other strings
 * freed on the calling thread (the pipeline thread that read the batch allocated them).
 *
 * The hook links this in place of the samSorter calls (-Wl,--wrap=new_samSorter,
 * --wrap=samSorter_processRead, --wrap=samSorter_processEnd, --wrap=samSorter_delete);
 * BSB_SAM_WRITER=0 keeps the reference's.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "bwa.h"
#include "bwamem_gpu.h"

typedef struct {
    bseq1_t **r;             /* the reads the step saw, in order */
    int64_t n, m;
    int active;
} so_batch_t;

static so_batch_t g_so;      /* kt_pipeline runs one output step at a time */

/* Blocks holding a whole batch's read strings (bseq_fast.c), by their first read's name: at most
 * the pipeline's batches in flight. */
#define SO_BLOCKS 16
static void *g_blocks[SO_BLOCKS];
static pthread_mutex_t g_blocks_mu = PTHREAD_MUTEX_INITIALIZER;

void sam_out_give_block(void *block)
{
    int k;
    pthread_mutex_lock(&g_blocks_mu);
    for (k = 0; k < SO_BLOCKS && g_blocks[k]; ++k) {}
    if (k < SO_BLOCKS) g_blocks[k] = block;
    pthread_mutex_unlock(&g_blocks_mu);
    if (k == SO_BLOCKS) {                  /* more batches in flight than the pipeline starts */
        fprintf(stderr, "[sam_out] too many read batches in flight\n");
        abort();
    }
}

/* 1 (and the entry dropped) when the batch whose first read's name is at p was one block */
static int so_take_block(void *p)
{
    int k, found = 0;
    pthread_mutex_lock(&g_blocks_mu);
    for (k = 0; k < SO_BLOCKS; ++k)
        if (p && g_blocks[k] == p) g_blocks[k] = 0, found = 1;
    pthread_mutex_unlock(&g_blocks_mu);
    return found;
}

int sam_out_enabled(void)
{
    static int on = -1;
    if (on < 0) {
        const char *e = getenv("BSB_SAM_WRITER");
        on = !(e && e[0] == '0');
    }
    return on;
}

static void so_push(bseq1_t *r)
{
    if (g_so.n == g_so.m) {
        g_so.m = g_so.m ? g_so.m * 2 : 1 << 16;
        g_so.r = (bseq1_t **)realloc(g_so.r, sizeof(bseq1_t *) * g_so.m);
        if (!g_so.r) {
            fprintf(stderr, "[sam_out] out of memory\n");
            abort();
        }
    }
    g_so.r[g_so.n++] = r;
}

void sam_out_begin(bseq1_t *first)
{
    g_so.n = 0;
    g_so.active = 1;
    so_push(first);
}

void sam_out_read(bseq1_t *read) { so_push(read); }

/* setUnmapped (bs_sorter.cpp:51-82): the unmapped record of a read, in a new string */
static char *so_unmapped(const bseq1_t *read)
{
    static const char fields[] = "*\t0\t0\t*\t*\t0\t0\t";
    const size_t ln = strlen(read->name);
    const int l = read->l_seq;
    char *s = (char *)malloc(ln + 2 * (size_t)l + 64), *p = s;
    int i;
    memcpy(p, read->name, ln), p += ln;
    *p++ = '\t';
    if (read->paired) {
        if (read->first) memcpy(p, "77\t", 3), p += 3;
        else memcpy(p, "141\t", 4), p += 4;
    } else memcpy(p, "4\t", 2), p += 2;
    memcpy(p, fields, sizeof fields - 1), p += sizeof fields - 1;
    for (i = 0; i < l; ++i) *p++ = "ACGTN"[(int)read->oseq[i]];
    *p++ = '\t';
    if (read->qual) memcpy(p, read->qual, (size_t)l), p += l;
    memcpy(p, "\tAS:i:0", 7), p += 7;
    memcpy(p, "\tYS:Z:WC\n", 9), p += 9;
    *p = 0;
    return s;
}

/* ---- the written records: measured and copied on threads ---- */

typedef struct {
    bseq1_t **out;           /* the reads written, in order */
    uint8_t *unmapped;       /* 1: rewritten as unmapped first */
    size_t *off;             /* byte offset of each record (off[n] = total) */
    char *buf;
    int64_t n, next;
    int phase;               /* 0: rewrite and measure, 1: copy (and free the record) */
} so_write_t;

/* seconds in each part of the output step, for BSB_GPU_STATS (sam_out_report) */
static double g_so_t[5];     /* decisions, measuring, copying, writing, freeing */

static double so_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + ts.tv_nsec * 1e-9;
}

void sam_out_report(FILE *fp)
{
    fprintf(fp, "[bsb_gpu] SAM output step: decisions %.3f s, measuring %.3f s, copying %.3f s, writing %.3f s, "
            "freeing the reads %.3f s\n", g_so_t[0], g_so_t[1], g_so_t[2], g_so_t[3], g_so_t[4]);
}

static void *so_worker(void *arg)
{
    so_write_t *W = (so_write_t *)arg;
    for (;;) {
        const int64_t a = __atomic_fetch_add(&W->next, 2048, __ATOMIC_RELAXED);
        int64_t i;
        if (a >= W->n) break;
        for (i = a; i < W->n && i < a + 2048; ++i) {
            bseq1_t *r = W->out[i];
            if (W->phase == 0) {
                if (W->unmapped[i]) {
                    free(r->sam);
                    r->sam = so_unmapped(r);
                }
                W->off[i] = r->sam ? strlen(r->sam) : 0;
            } else {
                if (W->off[i + 1] > W->off[i]) memcpy(W->buf + W->off[i], r->sam, W->off[i + 1] - W->off[i]);
                free(r->sam);        /* allocated by worker2's threads: freed here, in parallel */
                r->sam = 0;
            }
        }
    }
    return 0;
}

static void so_parallel(so_write_t *W, int phase)
{
    pthread_t th[32];
    long nc = sysconf(_SC_NPROCESSORS_ONLN);
    int t, nt = nc < 1 ? 1 : nc > 32 ? 32 : (int)nc, started = 0;
    W->phase = phase, W->next = 0;
    if (nt > (W->n + 2047) / 2048) nt = (int)((W->n + 2047) / 2048);
    for (t = 1; t < nt; ++t) {
        if (pthread_create(&th[t], 0, so_worker, W)) break;
        started = t;
    }
    so_worker(W);
    for (t = 1; t <= started; ++t) pthread_join(th[t], 0);
}

static void so_free_read(bseq1_t *r)
{
    free(r->name); free(r->comment);
    free(r->seq); free(r->qual);
    free(r->sam); free(r->oseq);
    r->name = r->comment = r->seq = r->qual = r->sam = r->oseq = 0;
}

/* processEnd and the reads before it: the reference's decisions over the batch, then the
 * records written, the BSStat counts printed and the reads freed. */
void sam_out_end(void)
{
    /* counters of the reference's samSorter (bs_sorter.h) */
    int wg2a = 0, wc2t = 0, cg2a = 0, cc2t = 0, unaligned = 0, bs_ambiguous = 0;
    int reads_observed = 0, alignments_observed = 0;
    int64_t i, k, n_out = 0;
    int64_t *g1 = (int64_t *)malloc(sizeof(int64_t) * (g_so.n + 1));
    int64_t *g2 = (int64_t *)malloc(sizeof(int64_t) * (g_so.n + 1));
    so_write_t W;
    memset(&W, 0, sizeof W);
    W.out = (bseq1_t **)malloc(sizeof(bseq1_t *) * (g_so.n + 1));
    W.unmapped = (uint8_t *)calloc((size_t)g_so.n + 1, 1);
    W.off = (size_t *)malloc(sizeof(size_t) * (g_so.n + 1));
    if (!g1 || !g2 || !W.out || !W.unmapped || !W.off) {
        fprintf(stderr, "[sam_out] out of memory\n");
        abort();
    }
    double t0 = so_now(), t1;
    /* one pass: groups of consecutive reads with one name (processRead, bs_sorter.cpp:37-51) */
    for (i = 0; i < g_so.n;) {
        const char *name = g_so.r[i]->name;
        int n1 = 0, n2 = 0, s1 = 0, s2 = 0, group;
        for (k = i; k < g_so.n && (k == i || strcmp(g_so.r[k]->name, name) == 0); ++k) {
            bseq1_t *r = g_so.r[k];                          /* bankRead (bs_sorter.cpp:126-135) */
            if (r->read_group == 0) s1 += r->alignment_score, g1[n1++] = k;
            else s2 += r->alignment_score, g2[n2++] = k;
        }
        group = s1 > s2 ? 0 : s1 < s2 ? 1 : 2;              /* pickReadGroup (:137-141) */
        ++reads_observed;                                   /* outputReads (:96-124) */
        {
            const int64_t *g = group == 1 ? g2 : g1;
            const int ng = group == 1 ? n2 : n1;
            int j;
            for (j = 0; j < ng; ++j) {
                bseq1_t *r = g_so.r[g[j]];
                if (group == 2) {
                    if (r->mapped) W.unmapped[n_out] = 1;
                    r->mapped = 0;
                    r->bs_conflict = 1;
                }
                ++alignments_observed;                      /* updateMappingStats (:84-94) */
                if (r->bs_conflict) ++bs_ambiguous;
                if (r->mapped == 0) ++unaligned;
                else if (r->mapped == 1) ++cg2a;
                else if (r->mapped == 2) ++cc2t;
                else if (r->mapped == 3) ++wg2a;
                else if (r->mapped == 4) ++wc2t;
                W.out[n_out++] = r;
            }
        }
        i = k;
    }
    W.n = n_out;
    t1 = so_now(), g_so_t[0] += t1 - t0, t0 = t1;
    so_parallel(&W, 0);
    t1 = so_now(), g_so_t[1] += t1 - t0, t0 = t1;
    {
        size_t acc = 0, len;
        for (i = 0; i < n_out; ++i) len = W.off[i], W.off[i] = acc, acc += len;
        W.off[n_out] = acc;
        W.buf = (char *)malloc(acc + 1);
        if (!W.buf) {
            fprintf(stderr, "[sam_out] out of memory\n");
            abort();
        }
        so_parallel(&W, 1);
        t1 = so_now(), g_so_t[2] += t1 - t0, t0 = t1;
        if (acc && fwrite(W.buf, 1, acc, stdout) != acc) {
            fprintf(stderr, "[sam_out] write error\n");
            exit(1);
        }
        t1 = so_now(), g_so_t[3] += t1 - t0, t0 = t1;
    }
    /* the reference prints the batch's counts from processEnd (bs_sorter_wrapper.cpp) */
    fprintf(stderr, "BSStat TotalReads: %d\n", reads_observed);
    fprintf(stderr, "BSStat TotalAlignments: %d\n", alignments_observed);
    fprintf(stderr, "BSStat W_C2T: %d\n", wc2t);
    fprintf(stderr, "BSStat W_G2A: %d\n", wg2a);
    fprintf(stderr, "BSStat C_C2T: %d\n", cc2t);
    fprintf(stderr, "BSStat C_G2A: %d\n", cg2a);
    fprintf(stderr, "BSStat Unaligned: %d\n", unaligned);
    fprintf(stderr, "BSStat BSAmbiguous: %d\n", bs_ambiguous);
    if (g_so.n && so_take_block(g_so.r[0]->name)) {    /* the batch's strings are one block */
        void *block = g_so.r[0]->name;
        for (i = 0; i < g_so.n; ++i) {
            bseq1_t *r = g_so.r[i];
            free(r->comment); free(r->sam);
            r->name = r->comment = r->seq = r->qual = r->sam = r->oseq = 0;
        }
        free(block);
    } else {
        for (i = 0; i < g_so.n; ++i) so_free_read(g_so.r[i]);
    }
    free(W.buf); free(W.out); free(W.unmapped); free(W.off); free(g1); free(g2);
    g_so_t[4] += so_now() - t0;
    g_so.n = 0;
    g_so.active = 0;
}
