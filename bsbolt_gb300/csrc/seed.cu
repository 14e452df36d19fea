// seed.cu -- SMEM seeding (mem_collect_intv) and suffix-array lookups on sm_103a.
//
// mem_collect_intv (bsbolt/External/BWA/bwamem.c:118-166) runs its three passes as
// independent work items of one persistent kernel (seed_kernel, state machine below):
//   pass 1  bwt_smem1 from every x (bwt.c:289-356), keep SMEMs >= min_seed_len;
//   pass 2  re-seed from the middle of SMEMs >= split_len with <= split_width hits
//           (a second launch: one item per such SMEM);
//   pass 3  bwt_seed_strategy1 (bwt.c:358-379) from every x;
// compact_seeds then sorts each read's seeds by info.  Equal info means the same
// substring and so the same interval, so the sort needs no tie rule.  The interval
// lists of bwt_smem1 live in a per-thread slice of device scratch (they are short in
// practice, but a repeat can make them as long as the read).  Every occurrence query
// reads one 32-byte sector of the occurrence array (fm_index.cuh).  An index of fewer
// than 2^32 - 2 rows runs the kernel on 32-bit intervals (96 registers, 5 blocks per SM,
// 16-byte list entries); a larger one on 64-bit intervals (128 registers, 4 blocks).
//
// bwt_sa (bwt.c:86-96) is one thread per suffix-array row: one load from the full
// suffix array when it is resident, else LF steps until a sampled row, each step
// one 32-byte sector.

#include "bsb_internal.cuh"
#include "fm_index.cuh"
#include "scan.cuh"

namespace {

constexpr int kSeedBlock = 128;

struct SeedOpt {
    int min_seed_len, split_len, split_width, max_mem_intv;
};

// The interval a seeding thread works with: bwtintv_t's fields in 64 bits (DevIntv), or, for
// an index of fewer than 2^32 - 2 rows, in 32 bits (SeedIntv32, info = qbeg << 16 | qend with
// read positions below 2^16), which halves the registers and the scratch bytes an interval
// costs.  IvT gives the info field's parts and the conversions to the output's DevIntv.
struct SeedIntv32 {
    uint32_t x0, x1, x2, info;
};

template <class IV> struct IvT;
template <> struct IvT<DevIntv> {
    using pos_t = uint64_t;
    static constexpr uint64_t kMaxRows = ~0ull;
    __device__ static uint64_t info(int qb, int qe) { return (uint64_t)(uint32_t)qb << 32 | (uint32_t)qe; }
    __device__ static int qbeg(const DevIntv &v) { return (int)(v.info >> 32); }
    __device__ static int qend(const DevIntv &v) { return (int)(uint32_t)v.info; }
    __device__ static DevIntv out(const DevIntv &v) { return v; }
    __device__ static DevIntv in(const DevIntv &v) { return v; }
};
template <> struct IvT<SeedIntv32> {
    using pos_t = uint32_t;
    static constexpr uint64_t kMaxRows = 0xfffffffdull;
    __device__ static uint32_t info(int qb, int qe) { return (uint32_t)qb << 16 | (uint32_t)qe; }
    __device__ static int qbeg(const SeedIntv32 &v) { return (int)(v.info >> 16); }
    __device__ static int qend(const SeedIntv32 &v) { return (int)(v.info & 0xffffu); }
    __device__ static DevIntv out(const SeedIntv32 &v)
    {
        DevIntv d;
        d.x0 = v.x0, d.x1 = v.x1, d.x2 = v.x2;
        d.info = (uint64_t)(v.info >> 16) << 32 | (v.info & 0xffffu);
        return d;
    }
    __device__ static SeedIntv32 in(const DevIntv &d)
    {
        SeedIntv32 v;
        v.x0 = (uint32_t)d.x0, v.x1 = (uint32_t)d.x1, v.x2 = (uint32_t)d.x2;
        v.info = (uint32_t)(d.info >> 32) << 16 | ((uint32_t)d.info & 0xffffu);
        return v;
    }
};

template <class IV>
__device__ __forceinline__ int seed_len(const IV &p)
{
    return IvT<IV>::qend(p) - IvT<IV>::qbeg(p);
}

// bwt_extend (bwt.c:262-275) of ik by the single base c: the reference computes all
// four extensions and its callers keep ok[c] only, so only that one is formed here.
template <class IV>
__device__ __forceinline__ IV extend_one(const DevFM &F, const IV &ik, bool is_back, int c)
{
    const uint64_t xf = is_back ? ik.x0 : ik.x1;     // x[!is_back]
    const uint64_t xb = is_back ? ik.x1 : ik.x0;     // x[is_back]
    const uint64_t x2 = ik.x2;
    Occ4 tk, tl;
    occ4_pair(F, xf - 1, xf - 1 + x2, tk, tl);        // in 64 bits whatever IV holds
    const uint64_t s0 = tl.c[0] - tk.c[0], s1 = tl.c[1] - tk.c[1], s2 = tl.c[2] - tk.c[2], s3 = tl.c[3] - tk.c[3];
    const uint64_t tkc = c == 0 ? tk.c[0] : c == 1 ? tk.c[1] : c == 2 ? tk.c[2] : tk.c[3];
    const uint64_t szc = c == 0 ? s0 : c == 1 ? s1 : c == 2 ? s2 : s3;
    const uint64_t above = c == 0 ? s1 + s2 + s3 : c == 1 ? s2 + s3 : c == 2 ? s3 : 0;   // bases > c
    const uint64_t l2c = l2_at(F, c);
    const uint64_t fw = l2c + 1 + tkc;
    const uint64_t bk = xb + (xf <= F.primary && xf + x2 - 1 >= F.primary) + above;
    IV o;
    o.x0 = (typename IvT<IV>::pos_t)(is_back ? fw : bk);
    o.x1 = (typename IvT<IV>::pos_t)(is_back ? bk : fw);
    o.x2 = (typename IvT<IV>::pos_t)szc;
    o.info = 0;
    return o;
}

// Seeding state machine.  Each loop iteration, every thread first runs its read's
// bookkeeping up to the next bwt_extend it needs (divergent, cheap), then all
// threads perform that extend together (converged, the expensive part), then apply
// its result.  The bookkeeping is mem_collect_intv (bwamem.c:118-166):
//   pass 1  bwt_smem1 from every x (bwt.c:289-356), keep SMEMs >= min_seed_len;
//   pass 2  re-seed from the middle of SMEMs >= split_len with <= split_width hits;
//   pass 3  bwt_seed_strategy1 (bwt.c:358-379) from every x;
// then the read's seeds are sorted by info (equal info = the same substring and so
// the same interval: no tie rule is needed, and the order seeds are found in does
// not matter -- compact_seeds sorts them).  Pass 2 depends only on pass 1's SMEMs,
// so it runs as a second launch with one work item per SMEM it re-seeds, in parallel
// with the other re-seeds instead of after them.  bwt_smem1 runs as:
//   FWD  extend ik forward from x, pushing ik whenever its size is about to change;
//        the pushes go down from the top of list A, so read upwards they are the
//        reference's reversed curr list;
//   BWD  one round per position i = x-1 .. -1: extend every prev entry backward by
//        q[i]; entries that fail may emit an SMEM (only while nothing has survived
//        this round), survivors are deduplicated by size into curr.
enum SeedState : int {
    kNeedRead, kP1X, kFwd, kFwdEnd, kBwdRound, kBwdEntry, kSmemDone, kP3X, kP3Fwd, kExit
};

// Launch control words: [0] next item of the first launch, [1] overflow (read + 1),
// [2] pass-2 items queued, [3] next item of the second launch, [4..5] the bwt_extend
// calls of both launches (uint64; each is one bwt_2occ4, two occurrence queries).
enum { kCtrlNext1 = 0, kCtrlOverflow = 1, kCtrlQueued = 2, kCtrlNext2 = 3, kCtrlExt = 4, kCtrlWords = 8 };

// Persistent: each thread takes work items from a counter.
//   mode 0: item r < n_reads runs pass 1 of read r and queues its pass-2 re-seeds;
//           item n_reads + r runs pass 3 of read r (independent of passes 1-2);
//   mode 1: item w runs the pass-2 re-seed queue[w] = (read, index of the SMEM).
// out holds, per read r, mult * (2*len(r) + 32) slots starting at mult * (2*(offs[r]-offs[0]) +
// 32*r): the first part_cap0(len, mult) for passes 1-2 (pass 2 appends with an atomic
// counter), the last part_cap1(len) (len/2 + 8: pass 3 finds at most one seed per
// min_seed_len + 1 >= 2 bases) for pass 3; count[2r + part] counts each part.  Passes 1-2
// have no such bound (every re-seed of a repeat can add SMEMs): a batch in which a read
// overflows runs again with mult doubled.
__device__ __host__ __forceinline__ int part_cap1(int len) { return len / 2 + 8; }
__device__ __host__ __forceinline__ int part_cap0(int len, int mult) { return mult * (2 * len + 32) - part_cap1(len); }
__device__ __host__ __forceinline__ int64_t part_base(int64_t rel_off, int r, int mult)
{
    return (int64_t)mult * (2 * rel_off + 32 * (int64_t)r);
}

// 4 blocks of 128 threads per SM on 64-bit intervals (128 registers), 5 on 32-bit ones.
template <class IV>
__global__ void __launch_bounds__(kSeedBlock, sizeof(IV) == sizeof(DevIntv) ? 4 : 5)
seed_kernel(DevFM F, SeedOpt opt, int mode, int n_reads, const uint8_t *__restrict__ seqs,
            const int64_t *__restrict__ offs, DevIntv *__restrict__ out, int *__restrict__ count,
            IV *__restrict__ scratch, int list_cap, int *__restrict__ ctrl, int2 *__restrict__ queue,
            int queue_cap, int mult)
{
    using T = IvT<IV>;
    using pos_t = typename T::pos_t;
    int *const next_item = ctrl + (mode ? kCtrlNext2 : kCtrlNext1);
    int *const overflow = ctrl + kCtrlOverflow;
    const int n_items = mode ? min(*(volatile int *)(ctrl + kCtrlQueued), queue_cap) : 2 * n_reads;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    IV *const listA = scratch + (size_t)tid * 3 * list_cap;          // forward pushes / curr and prev rounds
    IV *const listB = listA + list_cap;
    IV *const mem = listB + list_cap;                                // SMEMs of one bwt_smem1 call
    const int64_t base_off = offs[0];

    int st = kNeedRead;
    // read
    int r = 0, part = 0, len = 0, cap = 0, n = 0;
    const uint8_t *q = nullptr;
    DevIntv *dst = nullptr;
    // bwt_smem1
    int pass = 1, x = 0, i = 0, min_intv = 1, n_curr = 0, n_prev = 0, n_mem = 0, j = 0, c = 0, ret = 0;
    int last_mem_start = 0;
    pos_t last_x2 = 0;
    IV ik, p;
    IV *prev = listA, *curr = listB;
    // bwt_seed_strategy1
    int x0 = 0;
    // values loaded one step ahead, so their latency overlaps the extension in flight:
    // qi = q[i] (forward phases), qb = q[i] of the next backward round, pn = prev[j]
    int qi = 4, qb = 4;
    IV pn;
    ik.x0 = ik.x1 = ik.x2 = ik.info = 0;
    p = ik;
    pn = ik;
    unsigned n_ext = 0;

    for (;;) {
        // ---- bookkeeping up to the next extension (or the end of the work)
        IV e_ik;
        bool e_back = false;
        int e_c = 0;
        bool need = false;
        while (!need && st != kExit) {
            switch (st) {
            case kNeedRead: {
                // all pass-1 items first, then all pass-3 items: the warps that take
                // them hold items of similar length, so fewer lanes idle behind a long one
                const int w = atomicAdd(next_item, 1);
                if (w >= n_items) { st = kExit; break; }
                int k = 0;
                if (mode) {
                    const int2 it = queue[w];
                    r = it.x;
                    k = it.y;
                    part = 0;
                } else {
                    part = w >= n_reads;
                    r = part ? w - n_reads : w;
                }
                const int64_t o = offs[r];
                const int64_t len64 = offs[r + 1] - o;
                if (len64 < 0 || len64 > list_cap - 2) {    // outside the scratch the launch sized: refuse
                    count[2 * r + part] = 0;
                    atomicMax(overflow, r + 1);
                    break;
                }
                len = (int)len64;
                q = seqs + o;
                dst = out + part_base(o - base_off, r, mult) + (part ? part_cap0(len, mult) : 0);
                cap = part ? part_cap1(len) : part_cap0(len, mult);
                n = 0;
                if (mode) {                                  // re-seed in the middle of a long, rare SMEM
                    const DevIntv sm = dst[k];
                    pass = 2;
                    x = (int)(((sm.info >> 32) + (uint32_t)sm.info) >> 1);
                    min_intv = (int)sm.x2 + 1;
                    if (q[x] > 3) break;                     // bwt_smem1 returns at once: no SMEM
                    goto smem_start;
                }
                if (len < opt.min_seed_len || (part && opt.max_mem_intv <= 0)) {
                    count[2 * r + part] = 0;                 // mem_chain returns before seeding (bwamem.c:266)
                    break;
                }
                x = 0;
                st = part ? kP3X : kP1X;
                break;
            }
            case kP1X:
                if (x >= len) {                             // pass 1 done: queue the pass-2 re-seeds
                    if (n > cap) {
                        atomicMax(overflow, r + 1);
                        n = cap;
                    }
                    for (int t = 0; t < n; ++t) {
                        const DevIntv sm = dst[t];
                        const int start = (int)(sm.info >> 32), end = (int)(uint32_t)sm.info;
                        if (end - start < opt.split_len || sm.x2 > (uint64_t)opt.split_width) continue;
                        const int slot = atomicAdd(ctrl + kCtrlQueued, 1);
                        if (slot < queue_cap) queue[slot] = make_int2(r, t);
                        else atomicMax(overflow, r + 1);
                    }
                    count[2 * r] = n;
                    st = kNeedRead;
                    break;
                }
                if (q[x] > 3) { ++x; break; }
                pass = 1;
                min_intv = 1;
                goto smem_start;
            smem_start:
                if (min_intv < 1) min_intv = 1;
                ik = T::in(set_intv(F, q[x]));
                ik.info = T::info(0, x + 1);
                n_curr = 0;
                i = x + 1;
                qi = i < len ? q[i] : 4;
                st = kFwd;
                break;
            case kFwd:
                if (i < len && qi < 4) {
                    e_ik = ik; e_back = false; e_c = 3 - qi;
                    qi = i + 1 < len ? q[i + 1] : 4;         // for the next step
                    need = true;
                    break;
                }
                listA[list_cap - 1 - n_curr++] = ik;        // an N or the read end stops the match
                st = kFwdEnd;
                break;
            case kFwdEnd:
                prev = listA + list_cap - n_curr;            // reversed forward list
                curr = listB;
                n_prev = n_curr;
                ret = T::qend(prev[0]);
                n_mem = 0;
                i = x - 1;
                qb = i >= 0 ? q[i] : 4;
                st = kBwdRound;
                break;
            case kBwdRound:
                c = i < 0 ? -1 : (qb < 4 ? qb : -1);
                qb = i - 1 >= 0 ? q[i - 1] : 4;              // for the next round
                n_curr = 0;
                j = 0;
                pn = prev[0];
                st = kBwdEntry;
                break;
            case kBwdEntry:
                if (j >= n_prev) {
                    if (n_curr == 0) { st = kSmemDone; break; }
                    // this round's curr becomes the next prev; the list the old prev lived in
                    // (the forward pushes sit at the top of A) takes the next curr
                    IV *const was_prev = prev;
                    prev = curr;
                    curr = was_prev < listB ? listA : listB;
                    n_prev = n_curr;
                    --i;
                    st = kBwdRound;
                    break;
                }
                p = pn;
                if (j + 1 < n_prev) pn = prev[j + 1];       // for the next entry
                if (c >= 0) {
                    e_ik = p; e_back = true; e_c = c;
                    need = true;
                    break;
                }
                // no base to extend by: p cannot grow, and is maximal if nothing survived yet
                if (n_curr == 0 && (n_mem == 0 || i + 1 < last_mem_start)) {
                    IV m = p;
                    m.info |= T::info(i + 1, 0);
                    mem[n_mem++] = m;
                    last_mem_start = i + 1;
                }
                ++j;
                break;
            case kSmemDone:
                for (int t = 0; t < n_mem; ++t) {
                    const IV m = mem[t];
                    if (seed_len(m) >= opt.min_seed_len) {
                        if (pass == 1) {
                            if (n < cap) dst[n] = T::out(m);
                            ++n;
                        } else {                            // re-seeds of one read arrive from many threads
                            const int slot = atomicAdd(&count[2 * r], 1);
                            if (slot < cap) dst[slot] = T::out(m);
                            else atomicMax(overflow, r + 1);
                        }
                    }
                }
                if (pass == 1) { x = ret; st = kP1X; }
                else st = kNeedRead;
                break;
            case kP3X:
                if (x >= len) {                             // pass 3 done
                    if (n > cap) {
                        atomicMax(overflow, r + 1);
                        n = cap;
                    }
                    count[2 * r + 1] = n;
                    st = kNeedRead;
                    break;
                }
                if (q[x] > 3) { ++x; break; }
                ik = T::in(set_intv(F, q[x]));
                x0 = x;
                i = x + 1;
                qi = i < len ? q[i] : 4;
                st = kP3Fwd;
                break;
            case kP3Fwd:
                if (i >= len) { x = len; st = kP3X; break; }
                if (qi > 3) { x = i + 1; st = kP3X; break; }
                e_ik = ik; e_back = false; e_c = 3 - qi;
                qi = i + 1 < len ? q[i + 1] : 4;             // for the next step
                need = true;
                break;
            default:
                st = kExit;
                break;
            }
        }
        if (!__any_sync(BSB_FULL_MASK, need)) {
            if (st == kExit) break;
            continue;
        }
        n_ext += need;

        // ---- the extension, converged across the warp
        IV ok;
        if (need) ok = extend_one(F, e_ik, e_back, e_c);

        // ---- apply it
        if (!need) continue;
        switch (st) {
        case kFwd:
            if (ok.x2 != ik.x2) {
                listA[list_cap - 1 - n_curr++] = ik;
                if (ok.x2 < (pos_t)min_intv) { st = kFwdEnd; break; }
            }
            ik = ok;
            ik.info = T::info(0, i + 1);
            ++i;
            break;
        case kBwdEntry:
            if (ok.x2 < (pos_t)min_intv) {
                if (n_curr == 0 && (n_mem == 0 || i + 1 < last_mem_start)) {
                    IV m = p;
                    m.info |= T::info(i + 1, 0);
                    mem[n_mem++] = m;
                    last_mem_start = i + 1;
                }
            } else if (n_curr == 0 || ok.x2 != last_x2) {
                ok.info = p.info;
                curr[n_curr++] = ok;
                last_x2 = ok.x2;
            }
            ++j;
            break;
        case kP3Fwd:
            if (ok.x2 < (pos_t)opt.max_mem_intv && i - x0 >= opt.min_seed_len) {
                if (ok.x2 > 0) {                            // an empty interval is not kept (bwamem.c:160)
                    IV m = ok;
                    m.info = T::info(x0, i + 1);
                    if (n < cap) dst[n] = T::out(m);
                    ++n;
                }
                x = i + 1;
                st = kP3X;
                break;
            }
            ik = ok;
            ++i;
            break;
        default:
            break;
        }
    }
    if (n_ext) atomicAdd((unsigned long long *)(ctrl + kCtrlExt), (unsigned long long)n_ext);
}

// Seeds of read r in the two parts of its padded region (a part that overflowed holds
// its capacity; the launch reports the overflow).
__device__ __forceinline__ void part_counts(const int *__restrict__ count, const int64_t *__restrict__ offs, int r,
                                            int mult, int &na, int &nb)
{
    const int len = (int)(offs[r + 1] - offs[r]);
    na = min(count[2 * r], part_cap0(len, mult));
    nb = min(count[2 * r + 1], part_cap1(len));
}

// Seeds each read keeps (both parts, clamped to their caps), for the offset scan.
__global__ void read_totals(const int *__restrict__ count, const int64_t *__restrict__ offs, int n, int mult,
                            int *__restrict__ tot)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        int na, nb;
        part_counts(count, offs, r, mult, na, nb);
        tot[r] = na + nb;
    }
}

// Each read's seeds, sorted by info into the compact output (one block per read): an
// element's place is the number of elements with a smaller info, plus the number of
// equal ones before it (ks_introsort with intv_lt, bwamem.c:92-93; elements with equal
// info are equal, so the tie rule cannot show).
constexpr int kSortStage = 256, kCompactWarps = 4;
// One warp per read: the read's two parts merged into info order by rank (keys staged in
// the warp's slice of shared memory when they fit).
__global__ void __launch_bounds__(kCompactWarps * 32)
compact_seeds(const DevIntv *__restrict__ padded, const int64_t *__restrict__ offs, int n_reads, int mult,
              const int *__restrict__ count, const int64_t *__restrict__ out_off, DevIntv *__restrict__ out)
{
    __shared__ uint64_t keys[kCompactWarps][kSortStage];
    const int lane = threadIdx.x & 31, wb = threadIdx.x >> 5;
    uint64_t *key = keys[wb];
    const int64_t base_off = offs[0];
    for (int r = blockIdx.x * kCompactWarps + wb; r < n_reads; r += gridDim.x * kCompactWarps) {
        const int len = (int)(offs[r + 1] - offs[r]);
        const DevIntv *a = padded + part_base(offs[r] - base_off, r, mult);
        const DevIntv *b = a + part_cap0(len, mult);
        int na, nb;
        part_counts(count, offs, r, mult, na, nb);
        const int m = na + nb;
        DevIntv *dst = out + out_off[r];
        const bool staged = m <= kSortStage;
        __syncwarp();
        if (staged)
            for (int i = lane; i < m; i += 32) key[i] = (i < na ? a[i] : b[i - na]).info;
        __syncwarp();
        for (int i = lane; i < m; i += 32) {
            const DevIntv v = i < na ? a[i] : b[i - na];
            int rank = 0;
            for (int j = 0; j < m; ++j) {
                const uint64_t w = staged ? key[j] : (j < na ? a[j] : b[j - na]).info;
                rank += w < v.info || (w == v.info && j < i);
            }
            dst[rank] = v;
        }
    }
}

// Longest LF walk between sampled rows accepted: a valid index needs a few hundred
// steps at most (rows are sampled every sa_intv by row number); a corrupt one must not
// loop forever.
constexpr uint64_t kMaxWalk = 1ull << 20;

// bwt_sa: LF-walk to the nearest sampled row (bwt.c:53-59, 86-96), or one load when
// the full suffix array is resident.  Rows beyond seq_len are answered with
// (uint64_t)-2 and never walked; a walk longer than kMaxWalk with (uint64_t)-3.
__global__ void sa_kernel(DevFM F, const uint64_t *__restrict__ rows, int64_t n, uint64_t *__restrict__ pos)
{
    const uint64_t mask = (1ull << F.sa_shift) - 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t k = rows[i], steps = 0;
        if (k > F.seq_len) {
            pos[i] = ~(uint64_t)1;
            continue;
        }
        if (F.sa_full) {
            pos[i] = __ldg(F.sa_full + k);
            continue;
        }
        while ((k & mask) && steps < kMaxWalk) {
            ++steps;
            k = lf_step(F, k);
        }
        pos[i] = (k & mask) ? ~(uint64_t)2 : steps + __ldg(F.sa + (k >> F.sa_shift));
    }
}

// The full suffix array from the sampled one: sampled row s holds its sample, and the
// rows LF(s), LF^2(s), ... up to the next sampled row hold sa(s) - 1, sa(s) - 2, ...
// (bwt_sa's own walk, read backwards: every row's walk ends at the sampled row this
// fill starts from, so each row gets the value bwt_sa gives it).  Row 0 answers BWA's
// sample, (uint64_t)-1; the rows after it count down from seq_len.
__global__ void sa_fill_kernel(DevFM F, int64_t n_sa, uint64_t *__restrict__ full, int *__restrict__ failed)
{
    const uint64_t mask = (1ull << F.sa_shift) - 1;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_sa; t += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t s = (uint64_t)t << F.sa_shift;
        if (s > F.seq_len) continue;
        const uint64_t sv = F.sa[t];
        full[s] = sv;
        uint64_t v = s == 0 ? F.seq_len : sv, k = s;
        for (uint64_t step = 0;; ++step) {
            if (step >= kMaxWalk) {                      // not a valid index: the walk is kept
                atomicExch(failed, 1);
                break;
            }
            k = lf_step(F, k);
            if (!(k & mask)) break;                     // the next sampled row starts its own run
            full[k] = --v;
        }
    }
}

}  // namespace

size_t seed_scratch_bytes(int n_threads, int max_len)
{
    return (size_t)n_threads * 3 * (size_t)(max_len + 2) * sizeof(DevIntv);
}

// The 32-bit interval variant serves indexes of fewer than 2^32 - 2 rows.
static bool seed_narrow(uint64_t seq_len) { return seq_len < IvT<SeedIntv32>::kMaxRows; }

// Persistent seeding threads for an index of seq_len rows: as many as fit on the GPU at once
// (the variant the index runs sets the blocks per SM), no more than the reads need, and fewer
// when long reads would make the per-thread interval lists exceed ~1 GB of scratch.  The
// scratch of seed_scratch_bytes is sized by this count.
int seed_threads(int n_sm, int max_len, int n_reads, uint64_t seq_len)
{
    const bool narrow = seed_narrow(seq_len);
    static int resident[2] = {0, 0};
    if (!resident[narrow]) {
        int b = 0;
        const cudaError_t e =
            narrow ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, seed_kernel<SeedIntv32>, kSeedBlock, 0)
                   : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, seed_kernel<DevIntv>, kSeedBlock, 0);
        if (e != cudaSuccess || b < 1) b = 4;
        resident[narrow] = b;
    }
    const int res = resident[narrow];
    const size_t per_block = (size_t)kSeedBlock * 3 * (size_t)(max_len + 2) * sizeof(DevIntv);
    size_t blocks = (size_t)n_sm * res;
    const size_t want = ((size_t)2 * (n_reads > 0 ? n_reads : 1) + kSeedBlock - 1) / kSeedBlock;   // two items per read
    if (blocks > want) blocks = want;
    const size_t budget = (size_t)1 << 30;
    if (blocks * per_block > budget) blocks = budget / per_block;
    if (blocks < 1) blocks = 1;
    return (int)blocks * kSeedBlock;
}

// Pass-2 work items a batch can queue: at most one per SMEM of pass 1, i.e. per read
// position.
size_t seed_queue_entries(int64_t total_bases, int n_reads, int mult)
{
    return (size_t)mult * ((size_t)total_bases + (size_t)n_reads) + 64;
}

size_t seed_padded_entries(int64_t total_bases, int n_reads, int mult)
{
    return (size_t)mult * (2 * (size_t)total_bases + 32 * (size_t)n_reads);
}

cudaError_t seed_launch(const DevFM &F, int min_seed_len, float split_factor, int split_width, int max_mem_intv,
                        int n_reads, const uint8_t *d_seqs, const int64_t *d_offs, int max_len,
                        void *d_padded, int *d_count, int64_t *d_out_off, void *d_out,
                        void *d_lists, int *d_ctrl, void *d_queue, int64_t queue_cap, int *d_tot,
                        int64_t *d_scan_tmp, int mult, int n_sm, cudaStream_t st)
{
    SeedOpt o;
    o.min_seed_len = min_seed_len;
    o.split_len = (int)(min_seed_len * split_factor + .499);    // bwamem.c:122
    o.split_width = split_width;
    o.max_mem_intv = max_mem_intv;
    cudaError_t e = cudaMemsetAsync(d_ctrl, 0, kCtrlWords * sizeof(int), st);
    if (e != cudaSuccess) return e;
    const bool narrow = seed_narrow(F.seq_len);
    const int blocks = seed_threads(n_sm, max_len, n_reads, F.seq_len) / kSeedBlock;
    const int qcap = (int)(queue_cap < 0x7fffffff ? queue_cap : 0x7fffffff);
    for (int mode = 0; mode < 2; ++mode) {      // passes 1 and 3, then the pass-2 re-seeds
        if (narrow)
            seed_kernel<SeedIntv32><<<blocks, kSeedBlock, 0, st>>>(F, o, mode, n_reads, d_seqs, d_offs,
                                                                   (DevIntv *)d_padded, d_count, (SeedIntv32 *)d_lists,
                                                                   max_len + 2, d_ctrl, (int2 *)d_queue, qcap, mult);
        else
            seed_kernel<DevIntv><<<blocks, kSeedBlock, 0, st>>>(F, o, mode, n_reads, d_seqs, d_offs,
                                                                (DevIntv *)d_padded, d_count, (DevIntv *)d_lists,
                                                                max_len + 2, d_ctrl, (int2 *)d_queue, qcap, mult);
    }
    read_totals<<<n_sm * 4, 256, 0, st>>>(d_count, d_offs, n_reads, mult, d_tot);
    e = scan_i32_i64(d_tot, n_reads, d_out_off, d_scan_tmp, st);
    if (e != cudaSuccess) return e;
    const int cb = (int)((n_reads + kCompactWarps - 1) / kCompactWarps);
    compact_seeds<<<cb < n_sm * 16 ? cb : n_sm * 16, kCompactWarps * 32, 0, st>>>(
        (const DevIntv *)d_padded, d_offs, n_reads, mult, d_count, d_out_off, (DevIntv *)d_out);
    return cudaGetLastError();
}

cudaError_t sa_full_build(const DevFM &F, int64_t n_sa, uint64_t *full, int *failed, int n_sm, cudaStream_t st)
{
    const int64_t want = (n_sa + 255) / 256;
    const int blocks = (int)(want < (int64_t)n_sm * 32 ? want : (int64_t)n_sm * 32);
    sa_fill_kernel<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(F, n_sa, full, failed);
    return cudaGetLastError();
}

cudaError_t sa_launch(const DevFM &F, const uint64_t *d_rows, int64_t n, uint64_t *d_pos, int n_sm, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const int64_t want = (n + 255) / 256;
    const int blocks = (int)(want < (int64_t)n_sm * 16 ? want : (int64_t)n_sm * 16);
    sa_kernel<<<blocks, 256, 0, st>>>(F, d_rows, n, d_pos);
    return cudaGetLastError();
}
