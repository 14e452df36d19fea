/*
 * bsb_oracle_cigar.h -- CPU oracle for CIGAR / MD / XB generation.
 *
 * TEST INFRASTRUCTURE ONLY.  A plain-C restatement of the reference's
 * bwa_gen_cigar2 (bsbolt/External/BWA/bwa.c:199-351), ksw_global2
 * (ksw.c:504-606) and bns_get_seq (bntseq.c:413-434), used as the parity
 * checker for bsb_gen_cigar_batch and as its timed CPU baseline.  Nothing
 * in the product library links or calls it.  Its parity with the
 * reference is pinned by tests/golden/cigar_*.npz, produced by the
 * reference's own bwa_gen_cigar2 (oracle/Makefile.ref, make_golden.py).
 */
#ifndef BSB_ORACLE_CIGAR_H
#define BSB_ORACLE_CIGAR_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Job and result records: the layouts of bsb_cigar_job_t / bsb_cigar_out_t
 * in include/bsbgpu.h. */
typedef struct {
    int64_t rb, re, qoff, ooff;
    int32_t l_query, w;
} orc_cigar_job_t;

typedef struct {
    int32_t score, n_cigar, NM;
    int32_t cg_meth, cg_unmeth, ch_meth, ch_unmeth;
    int32_t status;
    int64_t off;
    int32_t bytes, pad;
} orc_cigar_out_t;

/* Status values (the same as BSB_CIGAR_* in bsbgpu.h). */
enum {
    ORC_CIGAR_OK = 0,         /* CIGAR words, then "MD\tXB:Z:calls\0" */
    ORC_CIGAR_REJECT = 1,     /* the reference returns no CIGAR (bwa.c:211, 214) */
    ORC_CIGAR_NO_MD = 2,      /* the 2-base context window bridges the strands: CIGAR only, NM -1 (bwa.c:266) */
    ORC_CIGAR_CLIPPED = 3,    /* the context window is clipped at an end of the doubled sequence:
                                 the reference reads past its buffer there */
    ORC_CIGAR_BAND_EXIT = 4   /* the traceback leaves the stored band: the reference reads
                                 unwritten backtrack cells there */
};

/* ksw_global2 (ksw.c:504-606) with m = 5.  Returns the score.  When cigar is
 * not NULL the CIGAR (reference encoding len<<4|op) is written there (room
 * for qlen + tlen words) and its length to *n_cigar; *band_exit is set when
 * the traceback reads outside the computed band. */
int orc_ksw_global2(int qlen, const uint8_t *query, int tlen, const uint8_t *target,
                    const int8_t mat[25], int o_del, int e_del, int o_ins, int e_ins, int w,
                    int *n_cigar, uint32_t *cigar, int *band_exit);

/* bwa_gen_cigar2 over a batch.  pac / opac are the 2-bit packed converted and
 * original references (l_pac bases each).  For job i the record goes to
 * out[i] and, for status OK / NO_MD, its bytes to blob + out[i].off (jobs
 * packed in order).  Returns the blob bytes used, or -1 when blob_cap is too
 * small.  n_threads pthreads. */
int64_t orc_gen_cigar_batch(const int8_t mat[25], int o_del, int e_del, int o_ins, int e_ins,
                            int64_t l_pac, const uint8_t *pac, const uint8_t *opac, int64_t crick_l,
                            int64_t n, const orc_cigar_job_t *jobs, const uint8_t *qbuf,
                            const uint8_t *obuf, orc_cigar_out_t *out, uint8_t *blob,
                            int64_t blob_cap, int n_threads);

/* bwa_gen_cigar2's score alone (bwa.c:199-244), as mem_patch_reg calls it (bwamem.c:432):
 * returns 0 where the reference leaves *score unset, else 1. */
int orc_gen_cigar2_score(const int8_t mat[25], int o_del, int e_del, int o_ins, int e_ins, int w_, int64_t l_pac,
                         const uint8_t *pac, int l_query, const uint8_t *query, int64_t rb, int64_t re, int *score);

#ifdef __cplusplus
}
#endif

#endif
