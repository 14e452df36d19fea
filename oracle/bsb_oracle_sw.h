/*
 * bsb_oracle_sw.h -- CPU oracle for the mate-rescue Smith-Waterman (ksw_align2).
 *
 * TEST INFRASTRUCTURE ONLY.  A plain-C restatement of the reference's striped
 * local alignment (bsbolt/External/BWA/ksw.c:48-365: ksw_qinit, ksw_u8,
 * ksw_i16, ksw_align2) -- the SIMD lanes written out as arrays, with the
 * reference's saturating 8-/16-bit arithmetic, its lazy-F loop and early exit,
 * its padded query columns, and its suboptimal-score bookkeeping -- used as
 * the parity checker for bsb_align2_batch.  Pinned by tests/golden/sw_*.npz,
 * produced by the reference's own ksw_align2.
 */
#ifndef BSB_ORACLE_SW_H
#define BSB_ORACLE_SW_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_KSW_XBYTE  0x10000
#define ORC_KSW_XSTOP  0x20000
#define ORC_KSW_XSUBO  0x40000
#define ORC_KSW_XSTART 0x80000

typedef struct { int32_t score, te, qe, score2, te2, tb, qb; } orc_kswr_t;    /* kswr_t, ksw.h:12-15 */

/* Job layout of bsb_sw_job_t (bsbgpu.h): query and target bytes (codes 0..4) in one
 * buffer; xtra = the KSW_X* flags and threshold as ksw_align2 takes them. */
typedef struct {
    int64_t qoff, toff;
    int32_t qlen, tlen, xtra, pad;
} orc_sw_job_t;

/* ksw_align2 (ksw.c:336-360) with m = 5; query and target are not modified. */
orc_kswr_t orc_ksw_align2(int qlen, const uint8_t *query, int tlen, const uint8_t *target, const int8_t mat[25],
                          int o_del, int e_del, int o_ins, int e_ins, int xtra);

void orc_align2_batch(int64_t n, const orc_sw_job_t *jobs, const uint8_t *seq, const int8_t mat[25], int o_del,
                      int e_del, int o_ins, int e_ins, orc_kswr_t *out, int n_threads);

#ifdef __cplusplus
}
#endif

#endif
