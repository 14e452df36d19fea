/*
 * ref_ksw_batch.c -- TEST INFRASTRUCTURE ONLY: the CPU baseline of the extension workload.
 *
 * Runs the reference's own ksw_extend2 (BSBolt's BWA fork, bsbolt/External/BWA/ksw.c:380-479,
 * compiled from its sources by oracle/Makefile.ref and linked here) over a batch of jobs laid
 * out as bsb_ext_job_t, on host threads that take chunks of jobs from a shared counter.  Only
 * bench.py's reference arm and CPU-baseline leg and the tests load it (oracle/_ref/libref_ksw.so).
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>

#include "ksw.h"

typedef struct {
    int64_t qoff, toff;
    int32_t qlen, tlen, h0, w, end_bonus, flags;
} rk_job_t;

typedef struct {
    int64_t n, next;
    const rk_job_t *jobs;
    const uint8_t *seq;
    const int8_t *mat;
    int o_del, e_del, o_ins, e_ins, zdrop;
    int32_t *out;
} rk_batch_t;

static void *rk_worker(void *arg)
{
    rk_batch_t *b = (rk_batch_t *)arg;
    for (;;) {
        int64_t lo = __atomic_fetch_add(&b->next, 1024, __ATOMIC_RELAXED), i;
        if (lo >= b->n) break;
        for (i = lo; i < b->n && i < lo + 1024; ++i) {
            const rk_job_t *j = &b->jobs[i];
            int32_t *o = b->out + 6 * i;
            int qle, tle, gtle, gscore, max_off;
            o[0] = ksw_extend2(j->qlen, b->seq + j->qoff, j->tlen, b->seq + j->toff, 5, b->mat, b->o_del, b->e_del,
                               b->o_ins, b->e_ins, j->w, j->end_bonus, b->zdrop, j->h0, &qle, &tle, &gtle, &gscore,
                               &max_off);
            o[1] = qle, o[2] = tle, o[3] = gtle, o[4] = gscore, o[5] = max_off;
        }
    }
    return 0;
}

/* out: n x 6 int32 (score, qle, tle, gtle, gscore, max_off), the reference's return values. */
int ref_ksw_batch(int64_t n, const void *jobs, const uint8_t *seq, const int8_t *mat, int o_del, int e_del,
                  int o_ins, int e_ins, int zdrop, int32_t *out, int n_threads)
{
    rk_batch_t b;
    pthread_t *tid;
    int t;
    if (n_threads < 1) n_threads = 1;
    b.n = n, b.next = 0, b.jobs = (const rk_job_t *)jobs, b.seq = seq, b.mat = mat;
    b.o_del = o_del, b.e_del = e_del, b.o_ins = o_ins, b.e_ins = e_ins, b.zdrop = zdrop, b.out = out;
    tid = (pthread_t *)malloc(sizeof(pthread_t) * n_threads);
    for (t = 0; t < n_threads; ++t) pthread_create(&tid[t], 0, rk_worker, &b);
    for (t = 0; t < n_threads; ++t) pthread_join(tid[t], 0);
    free(tid);
    return 0;
}
