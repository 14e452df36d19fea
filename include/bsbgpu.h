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
 * declared ksw.h:98-99) with one batch.  Host buffers; synchronous.
 * cells_out (optional, may be NULL) receives per job the number of DP cells
 * the reference visits (sum over rows of end-beg).  Requires qlen <= 1023,
 * 1 <= e_del, e_ins <= 65535, 0 <= o_del, o_ins <= 65535, matrix entries in
 * [-63, 63] and 0 < h0 <= 2^24 (the reference asserts h0 > 0); violations
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
 * also reports jobs the device rejected (qlen > 1023, h0 outside [1, 2^24],
 * ranges outside seq_bytes, nonzero flags) as BSB_EINVAL; those jobs' output
 * slots are left untouched. */
int bsb_sync(bsb_ctx *ctx);

/* Device time of the most recent extension batch on this context (CUDA
 * events on the context stream around its scheduling and extension
 * kernels), in milliseconds; valid after bsb_sync. */
float bsb_last_kernel_ms(const bsb_ctx *ctx);

/* ---- measurement helper (no reference counterpart) ---------------------- */

/* Measured 32-bit integer add+max throughput of this device, in tera
 * operations per second, counting each add and each max as one operation.
 * The roofline denominator for the integer-bound extension kernels. */
int bsb_probe_int_peak(bsb_ctx *ctx, double *tops, double *ms);

#ifdef __cplusplus
}
#endif
#endif /* BSBGPU_H */
