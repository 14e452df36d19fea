/*
 * bwamem_gpu.h -- the BWA-side glue of the GPU path.
 *
 * Compiled inside BSBolt's BWA fork (bsbolt/External/BWA), against its own
 * headers, and linked with libbsbgpu.so.  mem_align_batch_gpu() stands in for
 * the worker1 loop of mem_process_seqs (bwamem.c:1336,
 * `kt_for(opt->n_threads, worker1, &w, ...)`): it fills regs[0..n) exactly as
 * mem_align1_core (bwamem.c:1157-1195) would, so mem_pestat, worker2 and the
 * SAM writer run unchanged.
 */
#ifndef BWAMEM_GPU_H
#define BWAMEM_GPU_H

#include "bsbgpu.h"
#include "bwamem.h"

#ifdef __cplusplus
extern "C" {
#endif

/* bsb_align_opt_t from the reference's options. */
void mem_opt_to_bsb(const mem_opt_t *opt, bsb_align_opt_t *o);

/* Seeds, chains, extends and dedups n reads on the GPU (bsb_mem_align1_batch;
 * seqs[i].seq is the converted ASCII read, encoded to nt4 in place as
 * mem_align1_core does), then marks ALT regions per read.  regs[i].a is
 * malloc()ed (worker2 frees it).  Returns 0 or a BSB_E* code. */
int mem_align_batch_gpu(bsb_ctx *ctx, const mem_opt_t *opt, const bntseq_t *bns, const uint8_t *pac,
                        int n, bseq1_t *seqs, mem_alnreg_v *regs);
/* Batches so far whose first region buffer was too small (reads in a family of more
 * copies than a read has bases / 4, say) and ran again with the size the library gave. */
int64_t mem_align_regrown(void);

/* CIGAR pre-pass (bwa_gen_cigar2 on the GPU).  Called after mem_align_batch_gpu
 * and before worker2: runs bsb_gen_cigar_batch for the regions of the batch that
 * worker2 is expected to turn into SAM records or XA hits (score >= opt->T; which ones is
 * read off mem_mark_primary_se run on a copy of each read's regions with the id worker2
 * gives it, n_processed + i), with the first band mem_reg2aln tries
 * (bwamem.c:1219-1228), and keeps the records.  The glue's __wrap_bwa_gen_cigar2 (link
 * with -Wl,--wrap=bwa_gen_cigar2) answers a call whose job -- interval, band, query and
 * original-read bytes, scoring -- equals a kept record with a copy of it, and passes
 * every other call (band retries, mate-rescued regions, score-only calls, regions the
 * selection did not foresee) to the reference's own function, so the output is the
 * reference's either way.  The records live until the next pre-pass.  Returns 0 or a
 * BSB_E* code. */
int mem_gen_cigar_prepass_gpu(bsb_ctx *ctx, const mem_opt_t *opt, const bntseq_t *bns, int n, const bseq1_t *seqs,
                              const mem_alnreg_v *regs, int64_t n_processed);
/* Records kept by the last pre-pass, and calls answered from them since. */
void mem_gen_cigar_stats(int64_t *kept, int64_t *served);
/* Full bwa_gen_cigar2 calls (CIGAR and methylation outputs wanted) since the last pre-pass
 * that no kept record answered. */
int64_t mem_gen_cigar_passed(void);

/* Mate-rescue pre-pass (ksw_align2 on the GPU).  Called after mem_pestat and
 * before worker2 of a paired-end batch: for every pair it lists the ksw_align2
 * calls mem_sam_pe's rescue loop would make (bwamem_pair.c:265-274 choosing the
 * regions, mem_matesw bwamem_pair.c:111-154 the orientations, windows and
 * flags), with each mate's regions as they stand before any rescue, runs them
 * through bsb_align2_batch and keeps the results.  The glue's __wrap_ksw_align2
 * (link with -Wl,--wrap=ksw_align2) answers a call whose query, target, flags and
 * scoring equal a kept job's, and passes every other call (orientations that an
 * earlier rescue of the same pair reopened, mem_seed_sw's calls, mates over
 * BSB_SW_MAX_QLEN) to the reference's own function.  Nothing is kept for
 * single-end batches or with MEM_F_NO_RESCUE.  Returns 0 or a BSB_E* code. */
int mem_matesw_prepass_gpu(bsb_ctx *ctx, const mem_opt_t *opt, const bntseq_t *bns, const uint8_t *pac,
                           const mem_pestat_t pes[4], int n, const bseq1_t *seqs, const mem_alnreg_v *regs);
/* Jobs kept by the last mate-rescue pre-pass, and calls answered from them since. */
void mem_matesw_stats(int64_t *kept, int64_t *served);

/* bseq_read (bwa.c:73-143) with the same results, plain four-line FASTQ parsed with a line scan
 * and the entries built on threads; anything else goes to the reference's bseq_read, reached
 * as __real_bseq_read (link with -Wl,--wrap=bseq_read; bseq_fast.c). */
bseq1_t *bseq_read_fast(int64_t chunk_size, int *n_, void *ks1_, void *ks2_, int64_t *s, int conversion,
                        int undirectional, float substitution_proportion);

/* The output step of fastmap.c:process (samSorter, bs_sorter.cpp) with the same stdout bytes and
 * BSStat lines, records copied on threads and written once per batch (sam_out.c):
 * sam_out_begin(first read), sam_out_read per further read with a record, sam_out_end writes,
 * prints and frees (the records on the copying threads, a batch of read strings from
 * bseq_read_fast at once).  sam_out_enabled: 0 when BSB_SAM_WRITER=0. */
int sam_out_enabled(void);
void sam_out_begin(bseq1_t *first);
void sam_out_read(bseq1_t *read);
void sam_out_end(void);
/* the output step's time by part, one line (BSB_GPU_STATS) */
void sam_out_report(FILE *fp);
/* bseq_read_fast hands over a batch whose read strings (but comments) are one block starting at
 * the first read's name; sam_out_end frees it at once */
void sam_out_give_block(void *block);

#ifdef __cplusplus
}
#endif
#endif
