/*
 * bsb_oracle_chain.h -- CPU oracle types for chaining and chain extension.
 * TEST INFRASTRUCTURE ONLY (see bsb_oracle_chain.c).
 */
#ifndef BSB_ORACLE_CHAIN_H
#define BSB_ORACLE_CHAIN_H

#include <stdint.h>

#include "bsb_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { int64_t offset; int32_t len; int32_t is_alt; } orc_ann_t;

typedef struct {
    int64_t l_pac;               /* forward (Watson + Crick) length */
    int32_t n_seqs;
    const orc_ann_t *anns;
    const uint8_t *pac;          /* forward 2-bit text */
} orc_bns_t;

/* the mem_opt_t fields the path reads (bwamem.h:26-62) */
typedef struct {
    int32_t a, b, o_del, e_del, o_ins, e_ins, w, zdrop, pen_clip5, pen_clip3;
    int32_t min_seed_len, max_occ, max_chain_gap, min_chain_weight, max_chain_extend;
    float mask_level, drop_ratio, split_factor;
    int32_t split_width, max_mem_intv;
    int8_t mat[25];
    int8_t pad_[3];
    float mask_level_redun;      /* mem_sort_dedup_patch */
} orc_opt_t;

typedef struct { int64_t rbeg; int32_t qbeg, len, score, pad_; } orc_seed_t;   /* mem_seed_t */

typedef struct {                 /* mem_chain_t (bwamem.c:176-182) */
    int32_t n, rid, first, kept, w, is_alt;
    float frac_rep;
    int32_t seed_off;            /* index of the chain's first seed */
    int64_t pos;
} orc_chain_t;

typedef struct {                 /* the mem_alnreg_t fields mem_chain2aln sets (bwamem.h:64-82) */
    int64_t rb, re;
    int32_t qb, qe, rid, score, truesc, w, seedcov, seedlen0;
    float frac_rep;
    int32_t n_comp;              /* set by mem_sort_dedup_patch; 0 before */
} orc_reg_t;

int orc_mem_chain(const orc_bwt_t *bwt, const orc_bns_t *bns, const orc_opt_t *opt, int len,
                  const orc_intv_t *mem, int n_mem, orc_chain_t **chains, orc_seed_t **seeds, int *n_seeds);
int orc_mem_chain_flt(const orc_opt_t *opt, int n_chn, orc_chain_t *a, const orc_seed_t *seeds);
int orc_seed_sw_filter_applies(const orc_opt_t *opt, int l_query);
void orc_flt_chained_seeds(const orc_opt_t *opt, const orc_bns_t *bns, int l_query, const uint8_t *query,
                           int n_chn, orc_chain_t *a, orc_seed_t *seeds);
int orc_mem_chain2aln(const orc_opt_t *opt, const orc_bns_t *bns, int l_query, const uint8_t *query,
                      const orc_chain_t *c, const orc_seed_t *seeds, orc_reg_t *regs, int *n_regs, int max_regs,
                      int64_t *cells);

/* One batch of reads through seeds -> chains -> filter -> chain2aln (the
 * pre-dedup part of mem_align1_core, bwamem.c:1157-1180).  Outputs per read
 * (all offsets n_reads + 1 long): chains before filtering (chain0 / seeds0),
 * after filtering (chain1, sharing seeds0), and regions. */
typedef struct {
    orc_chain_t *chain0; int64_t *chain0_off;
    orc_seed_t *seeds0;  int64_t *seeds0_off;
    orc_chain_t *chain1; int64_t *chain1_off;
    orc_reg_t *regs;     int64_t *regs_off;
    int64_t cells;
} orc_align_out_t;

int orc_align_regs_batch(const orc_bwt_t *bwt, const orc_bns_t *bns, const orc_opt_t *opt, int n_reads,
                         const uint8_t *seqs, const int64_t *offs, orc_align_out_t *out, int n_threads);
void orc_align_out_free(orc_align_out_t *out);

#ifdef __cplusplus
}
#endif
#endif
