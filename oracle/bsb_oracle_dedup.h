/*
 * bsb_oracle_dedup.h -- CPU oracle for mem_sort_dedup_patch (the tail of
 * mem_align1_core).  TEST INFRASTRUCTURE ONLY (see bsb_oracle_dedup.c).
 */
#ifndef BSB_ORACLE_DEDUP_H
#define BSB_ORACLE_DEDUP_H

#include <stdint.h>

#include "bsb_oracle_chain.h"

#ifdef __cplusplus
extern "C" {
#endif

/* mem_sort_dedup_patch (bwamem.c:441-493) on one read's regions a[0..n) in place;
 * query: the read's nt4 bases; pac: the 2-bit forward text of l_pac bases.
 * Returns the number of regions kept. */
int orc_sort_dedup_patch(const orc_opt_t *opt, int64_t l_pac, const uint8_t *pac, const uint8_t *query, int n,
                         orc_reg_t *a);

/* The same per read of a batch: regs_in[in_off[r]..in_off[r+1]) -> regs_out[out_off[r]..). */
void orc_sort_dedup_batch(const orc_opt_t *opt, int64_t l_pac, const uint8_t *pac, int n_reads,
                          const uint8_t *seqs, const int64_t *offs, const orc_reg_t *regs_in, const int64_t *in_off,
                          orc_reg_t *regs_out, int64_t *out_off);

#ifdef __cplusplus
}
#endif
#endif
