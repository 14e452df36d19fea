/*
 * bsb_oracle.h -- CPU oracle for the bisulfite seed -> chain -> extend path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithms (BSBolt's BWA fork, bsbolt/External/BWA) used as the parity
 * checker for the CUDA path and as the timed CPU baseline.  Nothing in the
 * product library links or calls it.  Every function cites the reference
 * file:line it follows.  Parity of this restatement is pinned against the
 * reference itself (compiled from its own sources by oracle/Makefile.ref)
 * through the golden fixtures under tests/golden/.
 */
#ifndef BSB_ORACLE_H
#define BSB_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- banded extension (ksw.c:380-479) ---------------------------------- */

/* One call of the reference ksw_extend2 with m = 5.  Returns the best score;
 * the five out-params follow the reference.  *cells receives the number of
 * DP cells the reference's inner loop visits (sum over rows of end-beg). */
int orc_ksw_extend2(int qlen, const uint8_t *query, int tlen, const uint8_t *target,
                    const int8_t mat[25], int o_del, int e_del, int o_ins, int e_ins,
                    int w, int end_bonus, int zdrop, int h0,
                    int *qle, int *tle, int *gtle, int *gscore, int *max_off,
                    int64_t *cells);

/* Batch form over CSR-packed jobs (layout of bsb_ext_job_t in bsbgpu.h:
 * int64 qoff, int64 toff, int32 qlen, tlen, h0, w, end_bonus, pad).
 * out: 6 int32 per job (score,qle,tle,gtle,gscore,max_off).  cells may be
 * NULL.  Runs on n_threads pthreads; returns total cells. */
int64_t orc_ksw_batch(int64_t n, const void *jobs, const uint8_t *seq,
                      const int8_t mat[25], int o_del, int e_del, int o_ins, int e_ins,
                      int zdrop, int32_t *out, int64_t *cells, int n_threads);

/* ---- FM-index (bwt.h:46-80, bwt.c) -------------------------------------- */

typedef struct {
    uint64_t primary;
    uint64_t L2[5];
    uint64_t seq_len;
    uint64_t bwt_size;       /* in uint32 words */
    const uint32_t *bwt;     /* interleaved occurrence blocks, 16 words / 128 symbols */
    int sa_intv;
    uint64_t n_sa;
    const uint64_t *sa;      /* sa[0] == (uint64_t)-1 */
} orc_bwt_t;

typedef struct { uint64_t x[3], info; } orc_intv_t;

void orc_bwt_init(orc_bwt_t *b, uint64_t primary, const uint64_t L2_1to4[4],
                  const uint32_t *bwt, uint64_t bwt_size,
                  const uint64_t *sa, uint64_t n_sa, int sa_intv);
void orc_bwt_occ4(const orc_bwt_t *b, uint64_t k, uint64_t cnt[4]);
void orc_bwt_2occ4(const orc_bwt_t *b, uint64_t k, uint64_t l, uint64_t ck[4], uint64_t cl[4]);
void orc_bwt_extend(const orc_bwt_t *b, const orc_intv_t *ik, orc_intv_t ok[4], int is_back);
uint64_t orc_bwt_sa(const orc_bwt_t *b, uint64_t k);
int orc_bwt_smem1(const orc_bwt_t *b, int len, const uint8_t *q, int x, int min_intv,
                  orc_intv_t *mem, int *n_mem, int max_mem);
int orc_bwt_seed_strategy1(const orc_bwt_t *b, int len, const uint8_t *q, int x,
                           int min_len, int max_intv, orc_intv_t *mem);

/* Seeding options (subset of mem_opt_t, bwamem.h:26-62). */
typedef struct {
    int min_seed_len;      /* -k, 19 */
    float split_factor;    /* -r, 1.5 */
    int split_width;       /* 10 */
    int max_mem_intv;      /* 20 */
} orc_seed_opt_t;

/* mem_collect_intv (bwamem.c:118-166): all seeds of one read, sorted by info.
 * Returns the number of intervals written (or -1 if max_out is too small). */
int orc_collect_intv(const orc_bwt_t *b, const orc_seed_opt_t *opt, int len, const uint8_t *seq,
                     orc_intv_t *out, int max_out);

/* Batched collect_intv over reads packed as nt4 bytes with int64 offsets
 * (n+1 entries).  out_off receives n+1 offsets into out. */
int orc_collect_intv_batch(const orc_bwt_t *b, const orc_seed_opt_t *opt, int n,
                           const uint8_t *seqs, const int64_t *offs,
                           orc_intv_t *out, int64_t max_out, int64_t *out_off, int n_threads);

/* Batched SA lookups: pos[i] = bwt_sa(k[i]). */
void orc_bwt_sa_batch(const orc_bwt_t *b, int64_t n, const uint64_t *k, uint64_t *pos, int n_threads);

#ifdef __cplusplus
}
#endif
#endif
