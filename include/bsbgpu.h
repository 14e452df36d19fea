/*
 * bsbgpu.h -- C ABI of the GB300 (sm_103a) bisulfite seed/extend path.
 *
 * Plain C types only (pointers, sizes, fixed-width integers): callable from
 * C, C++ and ctypes.  Every entry point returns 0 on success or a negative
 * BSB_E* code; bsb_last_error() gives the message.  Nothing here exits or
 * aborts the process: the reference's err_fatal()/assert() paths become
 * error codes, and the caller (the BWA driver) decides whether to abort.
 *
 * Each entry point names the reference interface it stands in for
 * (BSBolt's BWA fork, bsbolt/External/BWA/...).
 */
#ifndef BSBGPU_H
#define BSBGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes ------------------------------------------------------- */
#define BSB_OK          0
#define BSB_EINVAL     -1   /* bad argument (size, pointer, option)            */
#define BSB_ECUDA      -2   /* a CUDA runtime call failed                     */
#define BSB_ENOMEM     -3   /* device or host allocation failed               */
#define BSB_EIO        -4   /* index file missing, short or inconsistent      */
#define BSB_ETIMEOUT   -5   /* a bounded device wait ran out                  */
#define BSB_ETOOLONG   -6   /* a sequence exceeds the supported length        */
#define BSB_ENOINDEX   -7   /* call needs an index and none is loaded         */
#define BSB_ECAPACITY  -8   /* batch larger than a fixed-size buffer allows   */

typedef struct bsb_ctx bsb_ctx;

/* Context: one CUDA device, one stream, device copies of the index.  A
 * context is not thread-safe; mem_process_seqs never runs concurrently with
 * itself (bsbolt/External/BWA/kthread.c:93-103), so one per process suffices. */
int  bsb_ctx_create(int device, bsb_ctx **out);
void bsb_ctx_destroy(bsb_ctx *ctx);
const char *bsb_last_error(const bsb_ctx *ctx);
const char *bsb_strerror(int code);
/* The CUDA stream every call of this context is ordered on (cudaStream_t). */
void *bsb_ctx_stream(bsb_ctx *ctx);

/* ---- banded extension: ksw_extend2 ------------------------------------- */

/* Scoring for a batch: the 5x5 matrix of bwa_fill_scmat (bwa.c:169-178) and
 * the affine gap / z-drop options of mem_opt_t (bwamem.h:27-31). */
typedef struct {
    int8_t  mat[25];
    int8_t  pad_[3];
    int32_t o_del, e_del, o_ins, e_ins;
    int32_t zdrop;
} bsb_ext_param_t;

/* One extension job: ksw_extend2(qlen, seq+qoff, tlen, seq+toff, 5, mat,
 * o_del, e_del, o_ins, e_ins, w, end_bonus, zdrop, h0, ...).  Query and
 * target bytes are nt4 codes 0..4 in one shared buffer. */
typedef struct {
    int64_t qoff, toff;
    int32_t qlen, tlen;
    int32_t h0, w, end_bonus;
    int32_t flags;            /* reserved, must be 0 */
} bsb_ext_job_t;

/* The reference's return value and five out-params, in call order. */
typedef struct {
    int32_t score, qle, tle, gtle, gscore, max_off;
} bsb_ext_out_t;

/* Replaces a loop of ksw_extend2 calls (bsbolt/External/BWA/ksw.c:380-479,
 * declared ksw.h:98-99) with one batch.  Host buffers; synchronous.  A batch
 * of 2^20 jobs or more runs in pieces whose host<->device copies overlap the
 * extension of the neighbouring pieces (best when the jobs' bytes are laid
 * out in job order in seq; the result never depends on it).
 * cells_out (optional, may be NULL) receives per job the number of DP cells
 * the reference visits (sum over rows of end-beg).  Requires qlen <= 1023,
 * 1 <= e_del, e_ins <= 65535, 0 <= o_del, o_ins <= 65535, matrix entries in
 * [-63, 63] and 0 < h0 <= 2^20 (the reference asserts h0 > 0); violations
 * return BSB_EINVAL / BSB_ETOOLONG before any device work. */
int bsb_extend_batch(bsb_ctx *ctx, const bsb_ext_param_t *param,
                     const bsb_ext_job_t *jobs, int64_t n_jobs,
                     const uint8_t *seq, int64_t seq_bytes,
                     bsb_ext_out_t *out, int64_t *cells_out);

/* Same, with every buffer already in device memory; asynchronous on the
 * context stream.  Jobs are binned by query-length tile and, within a bin,
 * issued most-expensive-first.  d_cost (optional, one int32 per job) is the
 * cost key used for that order -- e.g. a learned cell-count prediction; NULL
 * uses the plain bound qlen x min(tlen, qlen + w).  Results never depend on
 * the issue order. */
int bsb_extend_batch_device(bsb_ctx *ctx, const bsb_ext_param_t *param,
                            const bsb_ext_job_t *d_jobs, int64_t n_jobs,
                            const uint8_t *d_seq, int64_t seq_bytes,
                            const int32_t *d_cost,
                            bsb_ext_out_t *d_out, int64_t *d_cells);

/* Waits for the context stream.  After a bsb_extend_batch_device call it
 * also reports jobs the device rejected (qlen > 1023, h0 outside [1, 2^20],
 * ranges outside seq_bytes, nonzero flags) as BSB_EINVAL; those jobs' output
 * slots are left untouched. */
int bsb_sync(bsb_ctx *ctx);

/* Device time of the most recent extension batch on this context (CUDA
 * events on the context stream around its scheduling and extension
 * kernels), in milliseconds; valid after bsb_sync. */
float bsb_last_kernel_ms(const bsb_ctx *ctx);

/* ---- Extension tile shapes (no counterpart in the reference) -------------
 * A batched extension job runs on a tile of G lanes x C query columns per
 * lane (32/G jobs per warp); the tile map assigns a compiled shape to every
 * query length.  The shape changes the time, never a result.  The library
 * ships a default map measured on GB300; an autotuner (bsbolt_gb300.autotune)
 * can measure the shapes on the caller's own jobs and install its map. */
#define BSB_NUM_TILES 61
#define BSB_TILE_MAP_LEN 1025    /* entry [qlen + 1] for qlen = 0..1023; [0] unused */

/* Fills G[t], C[t] for the compiled shapes t < min(max, BSB_NUM_TILES);
 * returns BSB_NUM_TILES. */
int bsb_tile_shapes(int32_t *G, int32_t *C, int max);

/* Installs map (BSB_TILE_MAP_LEN entries, shape index per qlen + 1) for this
 * context's later extension batches; NULL restores the default map.  Every
 * entry [need], need = 1..1024, must name a shape with G*C >= need
 * (BSB_EINVAL otherwise, and the current map stays). */
int bsb_set_tile_map(bsb_ctx *ctx, const uint8_t *map, int n);

/* Device time of each shape's kernel in the context's most recent extension
 * batch (CUDA events around its launch on the stream it ran on), ms[t] for
 * t < min(n, BSB_NUM_TILES); 0 for shapes not launched.  Batches below 2^20
 * jobs run their shapes on four streams at once, so a shape's time there
 * includes sharing the GPU; a host batch extended in pieces reports its last
 * piece.  Valid after bsb_sync. */
int bsb_last_tile_ms(const bsb_ctx *ctx, float *ms, int n);

/* Copies the context's current tile map into map (n >= BSB_TILE_MAP_LEN);
 * ctx = NULL gives the built-in default map (no device needed). */
int bsb_get_tile_map(bsb_ctx *ctx, uint8_t *map, int n);

/* ---- FM-index (device resident) ----------------------------------------- */

/* The index arrays as bwa_idx_load leaves them in memory (bwa.c:363-524,
 * bwt.h:46-58): bwt = the interleaved occurrence array (bwt_size uint32
 * words), sa = the sampled suffix array with sa[0] = (uint64_t)-1, pac = the
 * forward bisulfite-converted 2-bit text (optional for seeding). */
typedef struct {
    uint64_t primary;
    uint64_t L2[5];              /* L2[0] = 0, L2[4] = seq_len */
    const uint32_t *bwt;
    uint64_t bwt_size;
    const uint64_t *sa;
    uint64_t n_sa;
    int32_t sa_intv;             /* power of two (bwt_cal_sa asserts it) */
    int32_t pad_;
    const uint8_t *pac;
    int64_t l_pac;
    int32_t n_seqs;              /* contig table (bntseq_t anns, bntseq.h:41-65): */
    int32_t pad2_;
    const int64_t *ann_offset;   /*   offset of each converted contig in the pac  */
    const int32_t *ann_len;      /*   and its length; needed by bsb_align_regs_batch */
} bsb_index_view_t;

/* Uploads an index the caller already holds (stands in for the host-side
 * index of bwa_idx_load, bwa.c:363-524).  Replaces any loaded index. */
int bsb_index_upload(bsb_ctx *ctx, const bsb_index_view_t *view);
/* Reads <prefix>.bwt/.sa/.ann/.pac (bwt_restore_bwt, bwt_restore_sa,
 * bwt.c:420-457) and uploads them.  BSB_EIO on a missing or short file. */
int bsb_index_load(bsb_ctx *ctx, const char *prefix);

/* Suffix array of the text bwa index sorts -- the 2-bit pac of l_pac bases, then its
 * reverse complement, then the '$' that sorts first (bwtindex.c; is.c / bwt_gen.c) -- sorted on
 * the GPU by prefix doubling over device radix sorts: sa[r] for r = 0 .. 2*l_pac (host buffer
 * of 2*l_pac + 1 int64), for the host's .bwt / .sa writer (bsbh_write_bwt_sa64).  Up to
 * 2*l_pac + 1 <= 2^32 - 1 suffixes (BSB_ETOOLONG beyond); takes ~33 bytes of device memory
 * per text symbol, freed on return.
 * No reference counterpart: bwa index sorts on the CPU. */
int bsb_build_suffix_array(bsb_ctx *ctx, const uint8_t *pac, int64_t l_pac, int64_t *sa);

/* The BWT and sampled suffix array of the same text, for texts of any length that fits device
 * memory (ranks are 64-bit): the suffixes are sorted by prefix doubling in chunks of at most
 * `chunk` suffixes (0: as many as the free device memory holds, ~44 bytes each, next to 9 bytes
 * per symbol for the text and the ranks).  Outputs (host buffers): bwt, (2*l_pac + 15)/16 words
 * of 2-bit symbols, 16 per word from the top bits, without the row of suffix 0 (bwt.h's
 * layout before the occurrence counts are interleaved); *primary, that row; sa[k] = SA[k *
 * sa_intv] for k < (2*l_pac + sa_intv)/sa_intv.  bsbolt_gb300.index.build_index writes
 * BWA's .bwt/.sa from them (bwtindex.c:256-321).  BSB_ENOMEM when one 5-symbol bucket of
 * suffixes does not fit a chunk.  No reference counterpart: bwa index sorts on the CPU. */
int bsb_build_bwt(bsb_ctx *ctx, const uint8_t *pac, int64_t l_pac, int sa_intv, int64_t chunk, uint32_t *bwt,
                  uint64_t *primary, uint64_t *sa);

/* Full suffix array (no counterpart in the reference).  An uploaded index also gets
 * every row's SA value in device memory (8 bytes per row), built from the sampled SA,
 * so each bwt_sa is one load instead of an LF walk; results are identical.  When it
 * does not fit, lookups walk as the reference does.  enable = 0 frees it (lookups
 * walk); 1 builds it again (BSB_ENOMEM when it does not fit). */
int bsb_index_full_sa(bsb_ctx *ctx, int enable);

/* ---- SMEM seeding: mem_collect_intv ------------------------------------- */

/* The seeding fields of mem_opt_t (bwamem.h:33-40). */
typedef struct {
    int32_t min_seed_len;        /* -k, 19 */
    float   split_factor;        /* -r, 1.5 */
    int32_t split_width;         /* 10 */
    int32_t max_mem_intv;        /* 20 */
} bsb_seed_opt_t;

/* bwtintv_t (bwt.h:60-62): x[0] forward start, x[1] reverse start, x[2]
 * size, info = qbeg << 32 | qend. */
typedef struct {
    uint64_t x[3];
    uint64_t info;
} bsb_intv_t;

/* Replaces mem_collect_intv (bwamem.c:118-166; bwt_smem1, bwt.c:289-356;
 * bwt_seed_strategy1, bwt.c:358-379) for a batch of reads: nt4 codes,
 * read r = seqs[offs[r] .. offs[r+1]).  out receives every read's seed list
 * in the reference's order (sorted by info), out_off[r] .. out_off[r+1]
 * (n_reads + 1 entries).  Reads shorter than min_seed_len get no seeds
 * (mem_chain, bwamem.c:266).  Reads longer than 1024 give BSB_ETOOLONG.  Each read
 * first gets 2*len + 32 seed slots; a batch in which a read's SMEMs and re-seeds need more
 * runs again with twice the slots, up to 64 times (bsb_mem_align1_batch and
 * bsb_align_regs_batch do the same). */
int bsb_seed_batch(bsb_ctx *ctx, const bsb_seed_opt_t *opt, int32_t n_reads,
                   const uint8_t *seqs, const int64_t *offs,
                   bsb_intv_t *out, int64_t max_out, int64_t *out_off);
/* Device-buffer form, asynchronous on the context stream.  d_offs must start
 * at 0; d_out must hold 2*total_bases + 32*n_reads entries; max_len bounds
 * every read length.  A read outside max_len is skipped and reported by
 * bsb_sync as BSB_ETOOLONG. */
int bsb_seed_batch_device(bsb_ctx *ctx, const bsb_seed_opt_t *opt, int32_t n_reads,
                          const uint8_t *d_seqs, const int64_t *d_offs, int64_t total_bases,
                          int32_t max_len, bsb_intv_t *d_out, int64_t *d_out_off);

/* Measurement helper (no reference counterpart): the bwt_extend calls -- each one
 * bwt_2occ4, i.e. two occurrence queries (bwt.c:189-220, 262-275) -- that the most
 * recent seeding batch of this context made, passes 1-3 together.  Waits for the
 * context stream. */
int bsb_last_seed_extensions(bsb_ctx *ctx, int64_t *n_ext);

/* ---- suffix-array lookup: bwt_sa ---------------------------------------- */

/* pos[i] = bwt_sa(bwt, rows[i]) (bwt.c:86-96) for every row; host buffers. */
int bsb_sa_batch(bsb_ctx *ctx, const uint64_t *rows, int64_t n, uint64_t *pos);
/* Device-buffer form; rows beyond seq_len give (uint64_t)-2. */
int bsb_sa_batch_device(bsb_ctx *ctx, const uint64_t *d_rows, int64_t n, uint64_t *d_pos);

/* ---- seeds -> chains -> regions: the pre-dedup part of mem_align1_core ---- */

/* The mem_opt_t fields the path reads (bwamem.h:26-62; BWA defaults in
 * mem_opt_init, bwamem.c:50-88). */
typedef struct {
    int32_t a, b, o_del, e_del, o_ins, e_ins, w, zdrop, pen_clip5, pen_clip3;
    int32_t min_seed_len, max_occ, max_chain_gap, min_chain_weight, max_chain_extend;
    float   mask_level, drop_ratio, split_factor;
    int32_t split_width, max_mem_intv;
    int8_t  mat[25];
    int8_t  pad_[3];
    float   mask_level_redun;    /* mem_sort_dedup_patch (bwa default 0.95) */
} bsb_align_opt_t;

/* The fields of mem_alnreg_t (bwamem.h:64-82) that mem_chain2aln sets; every
 * other field of the reference's struct is zero at that point.  n_comp is set
 * by mem_sort_dedup_patch (bsb_mem_align1_batch) and 0 before it. */
typedef struct {
    int64_t rb, re;
    int32_t qb, qe, rid, score, truesc, w, seedcov, seedlen0;
    float   frac_rep;
    int32_t n_comp;
} bsb_reg_t;

/* Replaces, for a batch of reads, the part of mem_align1_core
 * (bwamem.c:1157-1180) before mem_sort_dedup_patch: mem_collect_intv,
 * mem_chain (bwt_sa per sampled row, the chain tree), mem_chain_flt and
 * mem_chain2aln with its ksw_extend2 calls.  Reads are nt4 codes (already
 * converted, as mem_align1_core sees them); read r's regions, in the
 * reference's order, are regs[regs_off[r] .. regs_off[r+1]).  Needs an index
 * with pac and contig table.  Supports reads up to 1023 bp (longer ones return
 * BSB_ETOOLONG), with the seed-level Smith-Waterman filter of
 * mem_flt_chained_seeds (bwamem.c:602-619) run for every read length it applies
 * to, and indexes without ALT contigs (BSBolt writes none).  Host buffers;
 * synchronous.  When the batch has more
 * regions than max_regs (mem_chain samples up to max_occ rows per seed, so a
 * read in a large repeat family can have hundreds), nothing is written to regs,
 * regs_off is filled all the same (regs_off[n_reads] = the regions needed) and
 * the call returns BSB_ECAPACITY: call again with a buffer that large. */
int bsb_align_regs_batch(bsb_ctx *ctx, const bsb_align_opt_t *opt, int32_t n_reads,
                         const uint8_t *seqs, const int64_t *offs,
                         bsb_reg_t *regs, int64_t max_regs, int64_t *regs_off);

/* Replaces mem_align1_core (bwamem.c:1157-1195) for a batch of reads up to its
 * ALT marking: bsb_align_regs_batch followed by mem_sort_dedup_patch
 * (bwamem.c:441-493) per read -- the sort by end, the redundant regions
 * dropped (opt->mask_level_redun), colinear regions merged by mem_patch_reg
 * (bwamem.c:410-439, with its banded global alignment), the sort by score and
 * identical regions dropped.  Read r's regions, in the order mem_align1_core
 * returns them, are regs[regs_off[r] .. regs_off[r+1]); n_comp as the reference
 * sets it.  Marking regions on ALT contigs (bwamem.c:1189-1193) stays with the
 * caller (BSBolt's indexes have none).  Same limits, and the same BSB_ECAPACITY
 * answer to a short regs buffer, as bsb_align_regs_batch. */
int bsb_mem_align1_batch(bsb_ctx *ctx, const bsb_align_opt_t *opt, int32_t n_reads,
                         const uint8_t *seqs, const int64_t *offs,
                         bsb_reg_t *regs, int64_t max_regs, int64_t *regs_off);

/* Device time of the stages of the last bsb_align_regs_batch / bsb_mem_align1_batch
 * call, in ms, between marks recorded on the library's stream: [0] read upload and
 * seeding (mem_collect_intv), [1] suffix-array rows (bwt_sa), [2] chaining, chain
 * filter and the seed-level SW filter, [3] read order and mem_chain2aln, [4] region
 * compaction and mem_sort_dedup_patch, [5] region download.  Gaps where the stream
 * waits for the host (the two count read-backs) fall into the stage after them.
 * Writes min(n, BSB_ALIGN_STAGES) values; BSB_EINVAL before any batch. */
#define BSB_ALIGN_STAGES 6
int bsb_last_stage_ms(const bsb_ctx *ctx, float *ms, int n);

/* ---- CIGAR, MD and methylation strings: bwa_gen_cigar2 ------------------ */

/* Replaces bwa_gen_cigar2 (bwa.c:199-351; its ksw_global2, ksw.c:504-606) for a
 * batch of alignments, each called as mem_reg2aln calls it (bwamem.c:1228):
 * job = (rb, re) on the doubled sequence, the converted query (nt4) of
 * l_query bases at qbuf + qoff, the original read (nt4) at obuf + ooff (read
 * from its first base, as the reference does), band w_.  Needs an index with
 * pac and opac (bsb_index_upload_opac, or <prefix>.opac at bsb_index_load);
 * crick_l is bntseq_t.crick_l.  Per job, out[i] and, for status OK, the
 * reference's returned buffer -- n_cigar uint32 CIGAR words (len<<4|op), then
 * the NUL-terminated "MD\tXB:Z:calls" string -- at blob + out[i].off
 * (out[i].bytes bytes; jobs packed in order).  Host buffers; synchronous. */
#define BSB_CIGAR_OK 0          /* CIGAR words + MD/XB string */
#define BSB_CIGAR_REJECT 1      /* the reference returns no CIGAR (bwa.c:211, 214-215); bytes 0 */
#define BSB_CIGAR_NO_MD 2       /* the 2-base context window bridges the strands (bwa.c:264-266):
                                   CIGAR words only, NM -1, counts 0 */
#define BSB_CIGAR_CLIPPED 3     /* the context window is clipped at an end of the doubled sequence
                                   (rb < 2 or re > 2*l_pac - 2): the reference reads past its
                                   buffer there; no output */
#define BSB_CIGAR_BAND_EXIT 4   /* the traceback leaves the stored band, where the reference reads
                                   backtrack cells it never wrote; no output */
#define BSB_CIGAR_MAX_LEN 1024  /* longest query and reference interval of a job that is not rejected */
typedef struct {
    int64_t rb, re;
    int64_t qoff, ooff;
    int32_t l_query, w;
} bsb_cigar_job_t;
typedef struct {
    int32_t score, n_cigar, NM;
    int32_t cg_meth, cg_unmeth, ch_meth, ch_unmeth;
    int32_t status;
    int64_t off;
    int32_t bytes, pad_;
} bsb_cigar_out_t;

/* The original (unconverted) reference, 2-bit packed like the pac (bns->opac
 * as bwa_idx_load holds it).  Needs a loaded index with the same l_pac. */
int bsb_index_upload_opac(bsb_ctx *ctx, const uint8_t *opac, int64_t l_pac);
/* Uses opt's mat, o_del, e_del, o_ins, e_ins.  BSB_EINVAL when a job's bytes
 * lie outside qbuf / obuf or blob_cap is short (*blob_used then holds the bytes
 * needed); BSB_ETOOLONG for a job over BSB_CIGAR_MAX_LEN. */
int bsb_gen_cigar_batch(bsb_ctx *ctx, const bsb_align_opt_t *opt, int64_t crick_l, int32_t n,
                        const bsb_cigar_job_t *jobs, const uint8_t *qbuf, int64_t q_bytes,
                        const uint8_t *obuf, int64_t o_bytes, bsb_cigar_out_t *out,
                        uint8_t *blob, int64_t blob_cap, int64_t *blob_used);

/* ---- mate-rescue Smith-Waterman: ksw_align2 ----------------------------- */

/* Replaces a loop of ksw_align2 calls (ksw.c:336-360, declared ksw.h:59-60), as
 * mem_matesw makes them (bwamem_pair.c:150-151): local alignment of a query
 * against a target (codes 0..4 in one buffer) with the 5x5 matrix and gap
 * penalties of param (zdrop unused) and the KSW_X* flags and threshold in xtra
 * (KSW_XBYTE 0x10000, KSW_XSTOP 0x20000, KSW_XSUBO 0x40000, KSW_XSTART 0x80000).
 * out[i] = the reference's kswr_t, including its striped-SSE2 specifics: byte
 * lanes (16) with KSW_XBYTE, else 16-bit lanes (8), penalties broadcast at that
 * width, the lazy-F loop, padded query columns.  One case differs by design: a
 * byte-lane pass that saturates (score 255) with KSW_XSTART leaves tb = qb = -1,
 * where the reference profiles a zero-length query.  Needs a positive matrix
 * entry; at most 2^31 - 1 jobs per call, queries up to BSB_SW_MAX_QLEN.  Host
 * buffers; synchronous. */
#define BSB_SW_MAX_QLEN 1024
typedef struct {
    int64_t qoff, toff;
    int32_t qlen, tlen;
    int32_t xtra, pad_;
} bsb_sw_job_t;
typedef struct {
    int32_t score, te, qe, score2, te2, tb, qb;
} bsb_kswr_t;
int bsb_align2_batch(bsb_ctx *ctx, const bsb_ext_param_t *param, const bsb_sw_job_t *jobs, int64_t n_jobs,
                     const uint8_t *seq, int64_t seq_bytes, bsb_kswr_t *out);

/* ---- learned cost model for the extension scheduler ---------------------- */

/* No reference counterpart: BWA runs extensions in call order on CPU threads.
 * A 2 x 64 MLP (BF16 weights, FP32 accumulation) predicts log(1 + cells) of
 * an extension job; its prediction, as a cost key, only orders the issue of
 * jobs (bsb_extend_batch_device's d_cost) and never changes a result.  All
 * buffers are device memory; calls are asynchronous on the context stream. */
#define BSB_MLP_FEATURES 8
#define BSB_MLP_HIDDEN 64
#define BSB_MLP_PARAMS (64 * 8 + 64 * 64 + 64 + 64 + 64 + 1)
typedef struct {
    uint16_t w1[64 * 8];         /* BF16 bit patterns, row-major [out][in] */
    uint16_t w2[64 * 64];
    uint16_t w3[64];
    float b1[64], b2[64], b3;
} bsb_mlp_weights_t;

/* Eight features per job (see cost_mlp.cu): n x 8 floats. */
int bsb_cost_features(bsb_ctx *ctx, const bsb_ext_job_t *d_jobs, int64_t n, const uint8_t *d_seq,
                      int64_t seq_bytes, float *d_feat);
/* Predictions (log1p cells) and/or int32 cost keys (predicted cells); either may be NULL. */
int bsb_mlp_forward(bsb_ctx *ctx, const bsb_mlp_weights_t *d_w, const float *d_feat, int64_t n,
                    float *d_pred, int32_t *d_key);
/* Gradient of mean((y - target)^2) over n samples into d_grad[BSB_MLP_PARAMS]
 * (layout w1|w2|w3|b1|b2|b3), with the loss in d_grad[BSB_MLP_PARAMS].
 * Deterministic: each parameter's gradient is summed in sample order. */
int bsb_mlp_backward(bsb_ctx *ctx, const bsb_mlp_weights_t *d_w, const float *d_feat,
                     const float *d_target, int32_t n, float *d_grad);
/* One Adam step (beta 0.9 / 0.999) on FP32 master weights (BSB_MLP_PARAMS
 * floats, same layout) and moments; refreshes the BF16 weights. */
int bsb_mlp_adam(bsb_ctx *ctx, bsb_mlp_weights_t *d_w, float *d_master, float *d_m, float *d_v,
                 const float *d_grad, float lr, int32_t step);

/* ---- learned read order of the alignment batches ------------------------- */

/* No reference counterpart: BWA runs mem_chain2aln read by read on CPU threads.  Inside
 * bsb_align_regs_batch / bsb_mem_align1_batch one warp extends one read's chains at a
 * time, taking reads from a queue; by default the queue holds the reads with the most
 * chains first.  A 2 x 64 cost model (the bsb_mlp_* kernels above, BSB_MLP_FEATURES
 * features per read: read length, kept chains and their seeds, best chain weight, mean
 * seed offset, reverse-strand share, C+G content, the plain bound of the extension cells)
 * can order the queue by predicted DP cells instead.  The order never changes a result.
 *   bsb_read_cost_log(ctx, 1): later batches keep, per read, the features and the DP cells
 *     their ksw_extend2 calls visited (band retries included);
 *   bsb_last_read_costs: copies them out for the last batch (n_reads must match; host
 *     buffers of n_reads * BSB_MLP_FEATURES floats and n_reads int64);
 *   bsb_set_read_cost_model(ctx, d_w): order later batches by the model's prediction
 *     (weights in device memory, kept by the caller); NULL restores the chain-count order;
 *   bsb_set_read_order_keys(ctx, keys, n): order the next batch, which must hold n reads,
 *     by the caller's per-read keys (host int32, larger first, in the model's half-octave
 *     bins) -- e.g. the cells a log recorded, the order a perfect model would give, which
 *     bounds what any learned order can gain; used once, over the model; n = 0 clears. */
int bsb_read_cost_log(bsb_ctx *ctx, int enable);
int bsb_last_read_costs(bsb_ctx *ctx, int32_t n_reads, float *feat, int64_t *cells);
int bsb_set_read_cost_model(bsb_ctx *ctx, const bsb_mlp_weights_t *d_w);
int bsb_set_read_order_keys(bsb_ctx *ctx, const int32_t *keys, int32_t n);

/* ---- extension without any device allocation ---------------------------- */

/* No counterpart in the reference: BWA allocates freely on the host and has
 * no device.  This entry point is for callers that may not call cudaMalloc
 * -- code running under a host application whose memory manager owns all
 * device memory, or on a path where the implicit synchronisation of
 * cudaMalloc/cudaFree is not allowed.  It runs the same extension as
 * bsb_extend_batch_device, but its scheduling scratch is one fixed array of
 * the library's own device memory (about 2 MiB, held on every GPU that loads
 * the library until the process exits), so it calls no cudaMalloc, cudaFree
 * or other allocating routine and needs no context.
 *   - All buffers are the caller's device memory; the call is asynchronous
 *     on `stream` (a cudaStream_t; NULL = the legacy default stream) on the
 *     current device.
 *   - At most BSB_NOALLOC_MAX_JOBS jobs per call; a larger n_jobs returns
 *     BSB_ECAPACITY before any work is queued.
 *   - The first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress), also when n_jobs is 0; make that first call
 *     before any stream capture.  The extension kernels themselves are
 *     loaded by the CUDA runtime on their first launch, which takes device
 *     memory for their code: a warm-up batch that reaches the shapes and
 *     cell widths the later calls use (16-bit cells need penalties and
 *     scores as bsb_extend_batch allows them, max score <= 15) leaves
 *     nothing to load later.
 *   - Every shape of the library's default tile map is launched on every
 *     call (those with no jobs exit at once): the tile map is not chosen
 *     per batch.
 *   - Every call shares the array and it keeps the last call's contents
 *     (the launch clears what must start at zero).  Calls whose work
 *     overlaps on the GPU race on it: order them on one stream.
 *   - Jobs that fail the preconditions of bsb_extend_batch are skipped and
 *     their output slots left untouched, and nothing reports them: validate
 *     jobs as bsb_extend_batch does (qlen <= 1023, 0 < h0 <= 2^20, ranges
 *     inside seq_bytes, flags 0) before the call. */
#define BSB_NOALLOC_MAX_JOBS (1 << 18)
int bsb_extend_batch_noalloc(const bsb_ext_param_t *param, const bsb_ext_job_t *d_jobs,
                             int64_t n_jobs, const uint8_t *d_seq, int64_t seq_bytes,
                             bsb_ext_out_t *d_out, int64_t *d_cells, void *stream);

/* ---- measurement helper (no reference counterpart) ---------------------- */

/* Measured 32-bit integer add+max throughput of this device, in tera
 * operations per second, counting each add and each max as one operation.
 * The roofline denominator for the integer-bound extension kernels. */
int bsb_probe_int_peak(bsb_ctx *ctx, double *tops, double *ms);
/* The same on two 16-bit values per register (__viaddmax_s16x2): the peak of the
 * 16-bit cell kernels, four operations per instruction. */
int bsb_probe_int16x2_peak(bsb_ctx *ctx, double *tops, double *ms);

#ifdef __cplusplus
}
#endif
#endif /* BSBGPU_H */
