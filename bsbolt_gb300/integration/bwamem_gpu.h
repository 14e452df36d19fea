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

/* Seeds, chains and extends n reads (seqs[i].seq is the converted ASCII read,
 * encoded to nt4 in place as mem_align1_core does), then runs the reference's
 * own mem_sort_dedup_patch and ALT marking per read.  regs[i].a is malloc()ed
 * (worker2 frees it).  Returns 0 or a BSB_E* code. */
int mem_align_batch_gpu(bsb_ctx *ctx, const mem_opt_t *opt, const bntseq_t *bns, const uint8_t *pac,
                        int n, bseq1_t *seqs, mem_alnreg_v *regs);

#ifdef __cplusplus
}
#endif
#endif
