// bsb_internal.cuh -- shared declarations of the sm_103a bisulfite seed/extend library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/bsbgpu.h"

#define BSB_FULL_MASK 0xffffffffu

// Longest read the seeding kernels accept (bounds the per-thread interval lists).
#define BSB_SEED_MAX_LEN 1024
// Longest read the full seed-chain-extend batch accepts: its extensions fit the widest
// warp DP of chain2aln_kernel, 32 columns per lane (max_len + 1 <= 1024 columns).
#define BSB_ALIGN_MAX_LEN 1023
// Most pieces the host extension entry splits a batch into (copies overlap the extension).
#define BSB_MAX_CHUNKS 8
#define BSB_AUX_STREAMS 3

// Fork/join streams for the per-shape extension kernels of one batch.
struct KswStreams {
    cudaStream_t aux[BSB_AUX_STREAMS] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[BSB_AUX_STREAMS] = {};
};

struct bsb_ctx {
    int device = 0;
    int n_sm = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float last_kernel_ms = 0.f;
    int pending_ksw = 0;      // an extension batch was launched since the last bsb_sync
    std::string err;

    // growable device scratch owned by the context
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    // staging for the host-buffer entry points
    void *d_in = nullptr;
    size_t d_in_bytes = 0;
    void *d_out = nullptr;
    size_t d_out_bytes = 0;

    // device-resident FM-index (reference layout) and its scalars
    int has_index = 0;
    void *idx_bwt = nullptr, *idx_sa = nullptr, *idx_pac = nullptr;
    void *idx_sb = nullptr;       // superblock counts of the 64-symbol occurrence layout
    int idx_sym64 = 0;            // occurrence layout: 1 = 64 symbols per sector, 0 = 32
    void *idx_sa_full = nullptr;  // every row's SA value (built at upload when it fits), or NULL
    void *idx_opac = nullptr;     // original (unconverted) reference, 2-bit, for the methylation calls
    uint64_t primary = 0, seq_len = 0, n_sa = 0;
    uint64_t L2[5] = {0, 0, 0, 0, 0};
    int sa_intv = 0;
    int64_t l_pac = 0;
    // contig table (bntann1_t offsets and lengths) for chain extension
    void *idx_ann_off = nullptr, *idx_ann_len = nullptr;
    int n_seqs = 0;
    // seeding scratch (padded per-read seed lists, interval lists, counters)
    void *seed_scratch = nullptr;
    size_t seed_scratch_bytes = 0;
    int *seed_ctrl = nullptr;
    int64_t seed_regrown = 0;     // seeding batches run again with more seed slots per read
    // tile map of the batched extension (host copy; device copy only when it is not the default)
    uint8_t tile_map[BSB_TILE_MAP_LEN] = {};
    uint8_t *d_tile_map = nullptr;
    uint64_t map_tiles = 0;
    // per-shape device time of the last extension batch: tile_ev[2t], tile_ev[2t+1] are
    // recorded around shape t's kernel on the stream it runs on
    cudaEvent_t tile_ev[2 * BSB_NUM_TILES] = {};
    uint64_t last_tiles = 0;
    float tile_ms[BSB_NUM_TILES] = {};
    // extra streams: shape kernels of one batch run on `stream` and aux[] so that one
    // shape's tail overlaps the next; h2d/d2h carry the host entry's chunked copies
    KswStreams ms;
    cudaStream_t h2d = nullptr, d2h = nullptr;
    // host entry chunks: copy-in done, extension done, extension start/end marks
    cudaEvent_t chunk_ev[4 * BSB_MAX_CHUNKS] = {};
    int n_chunks = 0;
    // marks between the stages of the last alignment batch (bsb_last_stage_ms)
    cudaEvent_t stage_ev[BSB_ALIGN_STAGES + 1] = {};
    bool stage_valid = false;
    // chaining / chain-extension scratch
    void *arena0 = nullptr, *arena1 = nullptr, *arena2 = nullptr;
    size_t arena0_bytes = 0, arena1_bytes = 0, arena2_bytes = 0;
    // staging of the seed-level Smith-Waterman filter inside an alignment batch (the
    // batch's own reads and seeds occupy d_in / d_out meanwhile)
    void *flt_in = nullptr, *flt_out = nullptr, *flt_dev = nullptr;
    size_t flt_in_bytes = 0, flt_out_bytes = 0, flt_dev_bytes = 0;
    // learned read order of the alignment batches: the cost model (caller's device memory,
    // or NULL for the chain-count order), and the per-read features and extension cells of
    // the last batch when logging
    const void *read_model = nullptr;
    int read_log = 0, rc_n = 0;
    std::vector<int32_t> order_keys;   // per-read order keys for the next alignment batch
    void *rc_buf = nullptr;
    size_t rc_bytes = 0;
};

// bsb_align2_batch with explicit device staging buffers (grown as needed) in place of the
// context's d_in / d_out.
int bsb_align2_run(bsb_ctx *ctx, const bsb_ext_param_t *p, const bsb_sw_job_t *jobs, int64_t n, const uint8_t *seq,
                   int64_t seq_bytes, bsb_kswr_t *out, void **in_buf, size_t *in_bytes, void **out_buf,
                   size_t *out_bytes);

// SA lookups of device rows with the context's index (bwt_sa, bwt.c:86-96).
cudaError_t bsb_sa_launch_ctx(bsb_ctx *ctx, const uint64_t *d_rows, int64_t n, uint64_t *d_pos);

void bsb_index_release(bsb_ctx *ctx);

// Sets ctx->err and returns code.
int bsb_fail(bsb_ctx *ctx, int code, const char *fmt, ...);
// Maps a CUDA error to BSB_ECUDA with a message; returns 0 for cudaSuccess.
int bsb_cuda(bsb_ctx *ctx, cudaError_t e, const char *what);
// Ensures *buf holds at least bytes of device memory (grow-only).
int bsb_ensure(bsb_ctx *ctx, void **buf, size_t *cur, size_t bytes, const char *what);

// Device-side scoring for one extension batch.
struct KswParams {
    int8_t mat[25];
    int o_del, e_del, o_ins, e_ins, zdrop;
    int mat_max;
    int pack16;        // set by ksw_launch: the penalties allow 16-bit cells
};

// Launches the extension of n jobs (device buffers) on stream, scheduled by
// tile bin and cost key (d_cost, or the plain bound when NULL).
// scratch must hold ksw_scratch_bytes(n) bytes.  Returns a cudaError_t.
size_t ksw_scratch_bytes(int64_t n);
int ksw_max_qlen();
// Device word counting the jobs the last launch rejected (precondition failures).
int *ksw_rejected_counter(void *scratch);
// d_map: the tile map in device memory (BSB_TILE_MAP_LEN bytes), or NULL for
// the built-in default; tiles: bit t set = launch tile shape t (the shapes the
// batch's query lengths map to; a shape left out leaves its jobs unrun).
// tile_ev (optional, 2 * BSB_NUM_TILES events): per-shape timing marks as in bsb_ctx.
// ms (optional): run the shape kernels of batches below ksw_concurrent_below() jobs
// on st and ms->aux (joined back into st before ev1).
cudaError_t ksw_launch(const KswParams &P, const bsb_ext_job_t *d_jobs, int64_t n, int64_t seq_bytes,
                       const uint8_t *d_seq, const int32_t *d_cost, const uint8_t *d_map, uint64_t tiles,
                       bsb_ext_out_t *d_out, int64_t *d_cells, void *scratch, int n_sm, cudaStream_t st,
                       cudaEvent_t ev0, cudaEvent_t ev1, const cudaEvent_t *tile_ev = nullptr,
                       const KswStreams *ms = nullptr);
int64_t ksw_concurrent_below();
// The built-in tile map (host copy, BSB_TILE_MAP_LEN entries).
const uint8_t *ksw_default_tile_map();
// Shape of tile t; -1 if t is out of range.
int ksw_tile_shape(int t, int *G, int *C);
// Set of tile shapes a map uses (bit t).
uint64_t ksw_map_tiles(const uint8_t *map);

// (int)((double)num / e + 1.), the band caps of ksw.c:400-407, bwamem.c:627-628 and
// bwa.c:234-235, in integer arithmetic (e >= 1, |num| < 2^30): (num + e) / e truncated
// toward zero.  Where (num + e) / e
// is an integer both forms are exact; elsewhere it lies at least 1/e from every integer, far
// beyond the rounding of the two double operations, so truncation agrees.  (Double division
// runs on the GPU's slow fp64 pipe.)
__host__ __device__ __forceinline__ int band_cap(int num, int e) { return (num + e) / e; }

// bsb_seed_batch_device with mult times the per-read seed slots (d_out: seed_padded_entries(
// total, n, mult) entries); the caller reads the overflow word (seed_ctrl[1], read + 1) and
// runs the batch again with more slots, up to kSeedSlotMultMax.
constexpr int kSeedSlotMultMax = 64;
int bsb_seed_batch_device_m(bsb_ctx *ctx, const bsb_seed_opt_t *opt, int32_t n_reads, const uint8_t *d_seqs,
                            const int64_t *d_offs, int64_t total_bases, int32_t max_len, bsb_intv_t *d_out,
                            int64_t *d_out_off, int mult);
