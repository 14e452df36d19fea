// chain.cu -- seeds -> chains -> filtered chains -> alignment regions, on sm_103a.
//
// The pre-dedup part of mem_align1_core (bsbolt/External/BWA/bwamem.c:1157-1180)
// after seeding:
//   rows_count / rows_fill  the SA rows mem_chain samples per seed interval
//                           (bwamem.c:280-283), then sa_kernel (seed.cu) maps them
//                           to reference positions;
//   chain_kernel            one thread per read: mem_chain with the reference's
//                           B-tree of chains (kbtree.h, t = 5) so equal keys land
//                           where the reference puts them, then mem_chain_weight
//                           and mem_chain_flt with ks_introsort's exact order;
//   chain2aln_kernel        one warp per read: mem_chain2aln (bwamem.c:636-790),
//                           each ksw_extend2 run by the warp (ksw_core.cuh) on the
//                           read and the device 2-bit reference directly, so no
//                           reversed copies or target windows are materialised.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "bsb_internal.cuh"
#include "ksw_global.cuh"
#include "fm_index.cuh"
#include "ksw_core.cuh"
#include "scan.cuh"

size_t seed_padded_entries(int64_t total_bases, int n_reads, int mult);   // seed.cu

namespace {

constexpr int kBT = 5;                  // kbtree order for 40-byte keys in 512-byte nodes
constexpr int kBTMax = 2 * kBT - 1;

struct BtNode {
    int n, internal;
    int key[kBTMax];
    int child[kBTMax + 1];
};

struct ChainRec {                       // a chain while it is being built
    int64_t pos;                        // first seed's rbeg (the tree key)
    int64_t first_rbeg, last_rbeg;
    int first_qbeg, last_qbeg, last_len;
    int n, rid;
};

struct DevSeed {                        // mem_seed_t (bwamem.c:171-174)
    int64_t rbeg;
    int32_t qbeg, len, score, pad;
};

struct DevChain {                       // a kept chain, in mem_chain_flt's order
    int32_t n, rid, w, kept;
    int32_t seed_off, first;
    float frac_rep;
    int32_t pad;
};

struct AlnOpt {
    int a, o_del, e_del, o_ins, e_ins, w, zdrop, pen_clip5, pen_clip3;
    int min_seed_len, max_occ, max_chain_gap, min_chain_weight, max_chain_extend;
    float mask_level, drop_ratio;
};

struct DevBns {
    const int64_t *ann_offset;
    const int32_t *ann_len;
    int n_seqs;
    int64_t l_pac;
    const uint8_t *pac;
};

// ---------------------------------------------------------------- bns lookups

__device__ int pos2rid(const DevBns &B, int64_t pos_f)              // bntseq.c:364-379
{
    int left = 0, mid = 0, right = B.n_seqs;
    if (pos_f >= B.l_pac) return -1;
    while (left < right) {
        mid = (left + right) >> 1;
        if (pos_f >= B.ann_offset[mid]) {
            if (mid == B.n_seqs - 1) break;
            if (pos_f < B.ann_offset[mid + 1]) break;
            left = mid + 1;
        } else right = mid;
    }
    return mid;
}

__device__ __forceinline__ int64_t depos(const DevBns &B, int64_t pos, int &is_rev)
{
    is_rev = pos >= B.l_pac;
    return is_rev ? (B.l_pac << 1) - 1 - pos : pos;
}

__device__ int intv2rid(const DevBns &B, int64_t rb, int64_t re)    // bntseq.c:381-389
{
    int is_rev;
    if (rb < B.l_pac && re > B.l_pac) return -2;
    const int rid_b = pos2rid(B, depos(B, rb, is_rev));
    const int rid_e = rb < re ? pos2rid(B, depos(B, re - 1, is_rev)) : rid_b;
    return rid_b == rid_e ? rid_b : -1;
}

// base at position p of the forward-reverse text (bns_get_seq, bntseq.c:414-434)
__device__ __forceinline__ int text_base(const DevBns &B, int64_t p)
{
    if (p < B.l_pac) return __ldg(B.pac + (p >> 2)) >> ((~p & 3) << 1) & 3;
    p = (B.l_pac << 1) - 1 - p;
    return 3 - (__ldg(B.pac + (p >> 2)) >> ((~p & 3) << 1) & 3);
}

// ---------------------------------------------------------------- SA rows

__device__ __forceinline__ int rows_of(uint64_t x2, int max_occ, uint64_t &step)
{
    step = x2 > (uint64_t)max_occ ? x2 / (uint64_t)max_occ : 1;
    const uint64_t n = (x2 + step - 1) / step;                       // k = 0, step, ... < x2
    return (int)(n < (uint64_t)max_occ ? n : (uint64_t)max_occ);
}

__global__ void rows_count(const DevIntv *__restrict__ seeds, int64_t n, int max_occ, int *__restrict__ cnt)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t step;
        cnt[i] = rows_of(seeds[i].x2, max_occ, step);
    }
}

__global__ void rows_fill(const DevIntv *__restrict__ seeds, int64_t n, int max_occ, const int64_t *__restrict__ roff,
                          uint64_t *__restrict__ rows)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t step;
        const int m = rows_of(seeds[i].x2, max_occ, step);
        uint64_t *dst = rows + roff[i];
        for (int c = 0; c < m; ++c) dst[c] = seeds[i].x0 + (uint64_t)c * step;
    }
}

// ---------------------------------------------------------------- chaining

struct Bt {
    BtNode *nodes;
    int n_nodes, root;
    const ChainRec *ch;
    __device__ int64_t key(int c) const { return ch[c].pos; }
    __device__ int fresh()
    {
        BtNode &x = nodes[n_nodes];
        x.n = 0;
        x.internal = 0;
        return n_nodes++;
    }
    // lower bound stepped back unless equal (kbtree.h:116-130); r = 0 when equal
    __device__ int find(const BtNode &x, int64_t k, int &r) const
    {
        int begin = 0, end = x.n;
        if (x.n == 0) return -1;
        while (begin < end) {
            const int mid = (begin + end) >> 1;
            if (key(x.key[mid]) < k) begin = mid + 1;
            else end = mid;
        }
        if (begin == x.n) { r = 1; return x.n - 1; }
        const int64_t kb = key(x.key[begin]);
        r = k < kb ? -1 : (k > kb ? 1 : 0);
        if (r < 0) --begin;
        return begin;
    }
    __device__ int lower(int64_t k) const                             // kb_intervalp
    {
        int lo = -1, xi = root;
        for (;;) {
            const BtNode &x = nodes[xi];
            int r = 0;
            const int i = find(x, k, r);
            if (i >= 0 && r == 0) return x.key[i];
            if (i >= 0) lo = x.key[i];
            if (!x.internal) return lo;
            xi = x.child[i + 1];
        }
    }
    __device__ void split(int xi, int i, int yi)                      // kbtree.h:173-190
    {
        const int zi = fresh();
        BtNode &x = nodes[xi], &y = nodes[yi], &z = nodes[zi];
        z.internal = y.internal;
        z.n = kBT - 1;
        for (int j = 0; j < kBT - 1; ++j) z.key[j] = y.key[kBT + j];
        if (y.internal)
            for (int j = 0; j < kBT; ++j) z.child[j] = y.child[kBT + j];
        y.n = kBT - 1;
        for (int j = x.n; j >= i + 1; --j) x.child[j + 1] = x.child[j];
        x.child[i + 1] = zi;
        for (int j = x.n - 1; j >= i; --j) x.key[j + 1] = x.key[j];
        x.key[i] = y.key[kBT - 1];
        ++x.n;
    }
    __device__ void insert(int c)                                     // kbtree.h:191-223
    {
        const int64_t k = key(c);
        if (nodes[root].n == kBTMax) {
            const int si = fresh();
            nodes[si].internal = 1;
            nodes[si].child[0] = root;
            root = si;
            split(si, 0, nodes[si].child[0]);
        }
        int xi = root;
        for (;;) {
            BtNode &x = nodes[xi];
            int r;
            if (!x.internal) {
                const int i = find(x, k, r);
                for (int j = x.n - 1; j > i; --j) x.key[j + 1] = x.key[j];
                x.key[i + 1] = c;
                ++x.n;
                return;
            }
            int i = find(x, k, r) + 1;
            if (nodes[x.child[i]].n == kBTMax) {
                split(xi, i, x.child[i]);
                if (k > key(nodes[xi].key[i])) ++i;
            }
            xi = nodes[xi].child[i];
        }
    }
};

// ks_introsort (ksort.h:146-226) over an index array with the comparison lt(x, y):
// restated step for step, since records that compare equal keep the order it leaves.
template <class Lt>
struct KsSort {
    int *a;
    Lt lt;
    __device__ void insertsort(int s, int t)
    {
        for (int i = s + 1; i < t; ++i)
            for (int j = i; j > s && lt(a[j], a[j - 1]); --j) { int tmp = a[j]; a[j] = a[j - 1]; a[j - 1] = tmp; }
    }
    __device__ void combsort(int s, size_t n)
    {
        const double shrink_factor = 1.2473309501039786540366528676643;
        int do_swap;
        size_t gap = n;
        do {
            if (gap > 2) {
                gap = (size_t)(gap / shrink_factor);
                if (gap == 9 || gap == 10) gap = 11;
            }
            do_swap = 0;
            for (size_t i = 0; i + gap < n; ++i) {
                const int ii = s + (int)i, jj = ii + (int)gap;
                if (lt(a[jj], a[ii])) { int tmp = a[ii]; a[ii] = a[jj]; a[jj] = tmp; do_swap = 1; }
            }
        } while (do_swap || gap > 2);
        if (gap != 1) insertsort(s, s + (int)n);
    }
    __device__ void sort(int n, int *stk_l, int *stk_r, int *stk_d)
    {
        if (n < 1) return;
        if (n == 2) {
            if (lt(a[1], a[0])) { int tmp = a[0]; a[0] = a[1]; a[1] = tmp; }
            return;
        }
        int d;
        for (d = 2; 1ul << d < (unsigned long)n; ++d) ;
        int top = 0, s = 0, t = n - 1;
        d <<= 1;
        for (;;) {
            if (s < t) {
                if (--d == 0) {
                    combsort(s, (size_t)(t - s + 1));
                    t = s;
                    continue;
                }
                int i = s, j = t, k = i + ((j - i) >> 1) + 1;
                if (lt(a[k], a[i])) {
                    if (lt(a[k], a[j])) k = j;
                } else k = lt(a[j], a[i]) ? i : j;
                const int rp = a[k];
                if (k != t) { int tmp = a[k]; a[k] = a[t]; a[t] = tmp; }
                for (;;) {
                    do ++i; while (lt(a[i], rp));
                    do --j; while (i <= j && lt(rp, a[j]));
                    if (j <= i) break;
                    int tmp = a[i]; a[i] = a[j]; a[j] = tmp;
                }
                { int tmp = a[i]; a[i] = a[t]; a[t] = tmp; }
                if (i - s > t - i) {
                    if (i - s > 16) { stk_l[top] = s; stk_r[top] = i - 1; stk_d[top] = d; ++top; }
                    s = t - i > 16 ? i + 1 : t;
                } else {
                    if (t - i > 16) { stk_l[top] = i + 1; stk_r[top] = t; stk_d[top] = d; ++top; }
                    t = i - s > 16 ? i - 1 : s;
                }
            } else {
                if (top == 0) {
                    insertsort(0, n);
                    return;
                }
                --top;
                s = stk_l[top]; t = stk_r[top]; d = stk_d[top];
            }
        }
    }
};

// mem_chain_flt's order: chain weight, descending (bwamem.c:328-329)
struct FltLt {
    const int *w;
    __device__ bool operator()(int x, int y) const { return w[x] > w[y]; }
};

// One thread per read.  Per-read scratch is carved from arrays sized by the
// read's SA-row count R (a read never has more chains, seeds or tree nodes
// than rows).  Outputs the kept chains in mem_chain_flt's order and their
// seeds (in insertion order) at the read's row offset.
__global__ void __launch_bounds__(128)
chain_kernel(AlnOpt opt, DevBns B, int n_reads, const int64_t *__restrict__ read_off,
             const DevIntv *__restrict__ seeds, const int64_t *__restrict__ seed_off,
             const int64_t *__restrict__ row_off_of_seed, const uint64_t *__restrict__ pos,
             ChainRec *__restrict__ chains, BtNode *__restrict__ nodes, int *__restrict__ row_chain,
             int *__restrict__ iwork, DevSeed *__restrict__ out_seeds, DevChain *__restrict__ out_chains,
             int *__restrict__ n_chains, int *__restrict__ next)
{
    // reads in batch order: neighbouring threads' scratch (carved at the reads' row offsets)
    // shares cache lines; taking reads by row count instead ran 1.6 -> 3.8 ms on a 100 Mb batch
    for (;;) {
        const int r = atomicAdd(next, 1);
        if (r >= n_reads) break;
        const int len = (int)(read_off[r + 1] - read_off[r]);
        const int64_t s0 = seed_off[r], s1 = seed_off[r + 1];
        const int64_t R0 = row_off_of_seed[s0], R = row_off_of_seed[s1] - R0;
        n_chains[r] = 0;
        if (len < opt.min_seed_len || R == 0) continue;
        ChainRec *ch = chains + R0;
        BtNode *nd = nodes + R0;
        int *rc = row_chain + R0;
        // frac_rep (bwamem.c:271-278)
        int b = 0, e = 0, l_rep = 0;
        for (int64_t i = s0; i < s1; ++i) {
            const int sb = (int)(seeds[i].info >> 32), se = (int)(uint32_t)seeds[i].info;
            if (seeds[i].x2 <= (uint64_t)opt.max_occ) continue;
            if (sb > e) l_rep += e - b, b = sb, e = se;
            else e = e > se ? e : se;
        }
        l_rep += e - b;
        const float frac_rep = (float)l_rep / len;
        // mem_chain (bwamem.c:279-305)
        Bt bt;
        bt.nodes = nd;
        bt.n_nodes = 0;
        bt.ch = ch;
        bt.root = bt.fresh();
        int n_chn = 0;
        for (int64_t i = s0; i < s1; ++i) {
            const DevIntv p = seeds[i];
            const int slen = (int)((uint32_t)p.info - (uint32_t)(p.info >> 32));
            const int qbeg = (int)(p.info >> 32);
            const int64_t rlo = row_off_of_seed[i] - R0, rhi = row_off_of_seed[i + 1] - R0;
            for (int64_t k = rlo; k < rhi; ++k) {
                const int64_t rbeg = (int64_t)pos[R0 + k];
                rc[k] = -1;
                const int rid = intv2rid(B, rbeg, rbeg + slen);
                if (rid < 0) continue;
                bool to_add = true;
                if (n_chn > 0) {
                    const int lo = bt.lower(rbeg);
                    if (lo >= 0) {                               // test_and_merge (bwamem.c:203-227)
                        ChainRec &c = ch[lo];
                        const int64_t qend = c.last_qbeg + c.last_len, rend = c.last_rbeg + c.last_len;
                        if (rid != c.rid) {
                        } else if (qbeg >= c.first_qbeg && qbeg + slen <= qend && rbeg >= c.first_rbeg &&
                                   rbeg + slen <= rend) {
                            to_add = false;                      // contained: the seed is dropped
                        } else if ((c.last_rbeg < B.l_pac || c.first_rbeg < B.l_pac) && rbeg >= B.l_pac) {
                        } else {
                            const int64_t x = qbeg - c.last_qbeg, y = rbeg - c.last_rbeg;
                            if (y >= 0 && x - y <= opt.w && y - x <= opt.w && x - c.last_len < opt.max_chain_gap &&
                                y - c.last_len < opt.max_chain_gap) {
                                c.last_qbeg = qbeg; c.last_rbeg = rbeg; c.last_len = slen;
                                ++c.n;
                                rc[k] = lo;
                                to_add = false;
                            }
                        }
                    }
                }
                if (to_add) {
                    ChainRec &c = ch[n_chn];
                    c.pos = rbeg; c.first_rbeg = c.last_rbeg = rbeg;
                    c.first_qbeg = c.last_qbeg = qbeg; c.last_len = slen;
                    c.n = 1; c.rid = rid;
                    rc[k] = n_chn;
                    bt.insert(n_chn);
                    ++n_chn;
                }
            }
        }
        if (n_chn == 0) continue;
        // iwork layout (R ints each): order | seed start | weight | sort stack (3 x 64)
        int *order = iwork + R0 * 3, *sstart = order + R, *wgt = order + 2 * R;
        // in-order traversal (__kb_traverse); a t = 5 B-tree over < 2^31 keys is < 16 levels deep
        {
            int n_ord = 0;
            int stk_x[40], stk_i[40];
            int sp = 0;
            stk_x[0] = bt.root; stk_i[0] = 0;
            for (;;) {
                while (stk_x[sp] >= 0 && stk_i[sp] <= nd[stk_x[sp]].n) {
                    const BtNode &x = nd[stk_x[sp]];
                    stk_x[sp + 1] = x.internal ? x.child[stk_i[sp]] : -1;
                    stk_i[sp + 1] = 0;
                    ++sp;
                }
                --sp;
                if (sp >= 0) {
                    const int xi = stk_x[sp];
                    if (xi >= 0 && stk_i[sp] < nd[xi].n) order[n_ord++] = nd[xi].key[stk_i[sp]];
                    ++stk_i[sp];
                } else break;
            }
        }
        // seeds grouped by chain in insertion order: chain c's seeds start at sstart[c]
        for (int c = 0; c < n_chn; ++c) sstart[c] = 0;
        for (int64_t k = 0; k < R; ++k) if (rc[k] >= 0) ++sstart[rc[k]];
        {
            int acc = 0;
            for (int c = 0; c < n_chn; ++c) { const int v = sstart[c]; sstart[c] = acc; acc += v; }
        }
        DevSeed *sd = out_seeds + R0;
        {
            // place seeds; wgt[] counts per chain while placing
            for (int c = 0; c < n_chn; ++c) wgt[c] = 0;
            for (int64_t i = s0; i < s1; ++i) {
                const DevIntv p = seeds[i];
                const int slen = (int)((uint32_t)p.info - (uint32_t)(p.info >> 32));
                const int64_t rlo = row_off_of_seed[i] - R0, rhi = row_off_of_seed[i + 1] - R0;
                for (int64_t k = rlo; k < rhi; ++k) {
                    const int c = rc[k];
                    if (c < 0) continue;
                    DevSeed s;
                    s.rbeg = (int64_t)pos[R0 + k];
                    s.qbeg = (int)(p.info >> 32);
                    s.len = s.score = slen;
                    s.pad = 0;
                    sd[sstart[c] + wgt[c]++] = s;
                }
            }
        }
        // mem_chain_weight (bwamem.c:229-250) per chain, indexed by tree order
        for (int c = 0; c < n_chn; ++c) {
            const DevSeed *s = sd + sstart[c];
            const int n = ch[c].n;
            int64_t end = 0;
            int w = 0, tmp;
            for (int j = 0; j < n; ++j) {
                if (s[j].qbeg >= end) w += s[j].len;
                else if (s[j].qbeg + s[j].len > end) w += (int)(s[j].qbeg + s[j].len - end);
                end = end > s[j].qbeg + s[j].len ? end : s[j].qbeg + s[j].len;
            }
            tmp = w; w = 0; end = 0;
            for (int j = 0; j < n; ++j) {
                if (s[j].rbeg >= end) w += s[j].len;
                else if (s[j].rbeg + s[j].len > end) w += (int)(s[j].rbeg + s[j].len - end);
                end = end > s[j].rbeg + s[j].len ? end : s[j].rbeg + s[j].len;
            }
            w = w < tmp ? w : tmp;
            wgt[c] = w < (1 << 30) ? w : (1 << 30) - 1;
        }
        // mem_chain_flt (bwamem.c:331-389): drop light chains, sort by weight, mark kept
        int n = 0;
        for (int k = 0; k < n_chn; ++k)
            if (wgt[order[k]] >= opt.min_chain_weight) order[n++] = order[k];
        if (n == 0) continue;
        {
            int stk_l[64], stk_r[64], stk_d[64];
            KsSort<FltLt> fs{order, FltLt{wgt}};
            fs.sort(n, stk_l, stk_r, stk_d);
        }
        DevChain *oc = out_chains + R0;              // working copy, compacted at the end
        for (int k = 0; k < n; ++k) {
            const int c = order[k];
            oc[k].n = ch[c].n; oc[k].rid = ch[c].rid; oc[k].w = wgt[c];
            oc[k].kept = 0; oc[k].first = -1; oc[k].seed_off = sstart[c];
            oc[k].frac_rep = frac_rep; oc[k].pad = 0;
        }
        {
            // kept chain indices reuse rc[] (rows are no longer needed)
            int *kept = rc, n_kept = 0;
            oc[0].kept = 3;
            kept[n_kept++] = 0;
            for (int i = 1; i < n; ++i) {
                int large_ovlp = 0, k;
                const DevSeed *si = sd + oc[i].seed_off;
                const int bi = si[0].qbeg, ei = si[oc[i].n - 1].qbeg + si[oc[i].n - 1].len;
                for (k = 0; k < n_kept; ++k) {
                    const int j = kept[k];
                    const DevSeed *sj = sd + oc[j].seed_off;
                    const int bj = sj[0].qbeg, ej = sj[oc[j].n - 1].qbeg + sj[oc[j].n - 1].len;
                    const int b_max = bj > bi ? bj : bi, e_min = ej < ei ? ej : ei;
                    if (e_min > b_max) {                  // no ALT contigs: the is_alt test always passes
                        const int li = ei - bi, lj = ej - bj, min_l = li < lj ? li : lj;
                        if (e_min - b_max >= min_l * opt.mask_level && min_l < opt.max_chain_gap) {
                            large_ovlp = 1;
                            if (oc[j].first < 0) oc[j].first = i;
                            if (oc[i].w < oc[j].w * opt.drop_ratio && oc[j].w - oc[i].w >= opt.min_seed_len << 1)
                                break;
                        }
                    }
                }
                if (k == n_kept) {
                    kept[n_kept++] = i;
                    oc[i].kept = large_ovlp ? 2 : 3;
                }
            }
            for (int i = 0; i < n_kept; ++i)
                if (oc[kept[i]].first >= 0) oc[oc[kept[i]].first].kept = 1;
            int i, k = 0;
            for (i = 0; i < n; ++i) {
                if (oc[i].kept == 0 || oc[i].kept == 3) continue;
                if (++k >= opt.max_chain_extend) break;
            }
            for (; i < n; ++i)
                if (oc[i].kept < 3) oc[i].kept = 0;
            for (i = k = 0; i < n; ++i)
                if (oc[i].kept != 0) oc[k++] = oc[i];
            n_chains[r] = k;
        }
    }
}

// ---------------------------------------------------------------- chain2aln

// Query base j and target base i of one extension: q(j) = read[q0 + qdir*j],
// t(i) = text base at t0 + tdir*i.  Left extensions run on both reversed,
// as the reference's reversed copies do (bwamem.c:721-724).
struct ReadRefAcc {
    const uint8_t *read;
    int q0, qdir;
    int64_t t0;
    int tdir;
    DevBns B;
    __device__ __forceinline__ int q(int j) const { return read[q0 + qdir * j]; }
    __device__ __forceinline__ int t(int i) const { return text_base(B, t0 + (int64_t)tdir * i); }
};

__device__ __forceinline__ int cal_max_gap(const AlnOpt &o, int qlen)         // bwamem.c:625-632
{
    const int l_del = band_cap(qlen * o.a - o.o_del, o.e_del);
    const int l_ins = band_cap(qlen * o.a - o.o_ins, o.e_ins);
    int l = l_del > l_ins ? l_del : l_ins;
    l = l > 1 ? l : 1;
    return l < o.w << 1 ? l : o.w << 1;
}

template <int C>
__device__ KswResult run_ext(const KswParams &P, int qlen, int tlen, int h0, int w, int eb, const ReadRefAcc &acc,
                             int lane)
{
    return ksw_warp<C>(P, qlen, tlen, h0, w, eb, acc, lane);
}

// A warp tile (C columns per lane) that holds qlen + 1 columns; a kernel compiled for
// reads of at most 32 * MaxC - 1 bases only instantiates C <= MaxC.
template <int MaxC>
__device__ KswResult extend_any(const KswParams &P, int qlen, int tlen, int h0, int w, int eb, const ReadRefAcc &acc,
                                int lane)
{
    // One width per kernel where it can be: each width is a fully unrolled copy of the
    // DP, and the warps of an SM run extensions of every length at once, so extra copies
    // cost more in instruction-cache misses than the columns a tighter fit saves
    // (measured on GB300: one 8-column copy beat {1, 2, 4, 8} by 20 % on a 100 Mb
    // reference with repeats and 2x150 reads, and by 2 % on a 2 Mb one with 2x100).
    const int need = (qlen + 32) >> 5;
    if constexpr (MaxC <= 8) {
        return run_ext<MaxC>(P, qlen, tlen, h0, w, eb, acc, lane);
    } else if constexpr (MaxC <= 16) {
        if (need <= 8) return run_ext<8>(P, qlen, tlen, h0, w, eb, acc, lane);
        return run_ext<16>(P, qlen, tlen, h0, w, eb, acc, lane);
    } else {                 // reads of 512-1023 bases: extensions past 511 columns need 32 per lane
        if (need <= 8) return run_ext<8>(P, qlen, tlen, h0, w, eb, acc, lane);
        if (need <= 16) return run_ext<16>(P, qlen, tlen, h0, w, eb, acc, lane);
        return run_ext<32>(P, qlen, tlen, h0, w, eb, acc, lane);
    }
}

// One warp per read.  regs: the read's region slots start at its row offset.
// MaxC = 4, 5, 8 serve batches whose reads are at most 127, 159, 255 bases long (one DP
// copy of that width), 16 every read the batch accepts; the 4- and 5-column variants are
// held to 4 blocks (16 warps) per SM, the 8-column one to 3.
template <int MaxC>
__global__ void __launch_bounds__(128, MaxC <= 5 ? 4 : MaxC <= 8 ? 3 : 1)
chain2aln_kernel(AlnOpt opt, KswParams P, DevBns B, int n_reads, const uint8_t *__restrict__ reads,
                 const int64_t *__restrict__ read_off, const int64_t *__restrict__ seed_off,
                 const int64_t *__restrict__ row_off_of_seed, const DevSeed *__restrict__ seeds,
                 const DevChain *__restrict__ chains, const int *__restrict__ n_chains, uint64_t *__restrict__ srt_buf,
                 bsb_reg_t *__restrict__ regs, int *__restrict__ n_regs, int *__restrict__ next,
                 const int *__restrict__ order, int64_t *__restrict__ read_cells)
{
    const int lane = threadIdx.x & 31;
    for (;;) {
        int k = 0;
        if (lane == 0) k = atomicAdd(next, 1);
        k = __shfl_sync(BSB_FULL_MASK, k, 0);
        if (k >= n_reads) break;
        const int r = order[k];
        const int64_t R0 = row_off_of_seed[seed_off[r]];
        const int nc = n_chains[r];
        const int l_query = (int)(read_off[r + 1] - read_off[r]);
        const uint8_t *query = reads + read_off[r];
        const DevSeed *sd = seeds + R0;
        const DevChain *chn = chains + R0;
        bsb_reg_t *av = regs + R0;
        uint64_t *srt = srt_buf + R0;
        int nav = 0;
        long long cells = 0;           // DP cells of the read's ksw_extend2 calls, band retries included
        const int64_t l_pac = B.l_pac;
        for (int ci = 0; ci < nc; ++ci) {
            const DevChain c = chn[ci];
            const DevSeed *cs = sd + c.seed_off;
            if (c.n == 0) continue;
            // the widest target span any seed can use (bwamem.c:646-661)
            int64_t rmax0 = l_pac << 1, rmax1 = 0;
            for (int i = 0; i < c.n; ++i) {
                const DevSeed t = cs[i];
                const int64_t b = t.rbeg - (t.qbeg + cal_max_gap(opt, t.qbeg));
                const int64_t e = t.rbeg + t.len + ((l_query - t.qbeg - t.len) + cal_max_gap(opt, l_query - t.qbeg - t.len));
                rmax0 = rmax0 < b ? rmax0 : b;
                rmax1 = rmax1 > e ? rmax1 : e;
            }
            rmax0 = rmax0 > 0 ? rmax0 : 0;
            rmax1 = rmax1 < l_pac << 1 ? rmax1 : l_pac << 1;
            if (rmax0 < l_pac && l_pac < rmax1) {
                if (cs[0].rbeg < l_pac) rmax1 = l_pac;
                else rmax0 = l_pac;
            }
            {   // bns_fetch_seq's clip to the contig of the first seed (bntseq.c:436-461)
                int is_rev;
                const int rid = pos2rid(B, depos(B, cs[0].rbeg, is_rev));
                int64_t far_beg = B.ann_offset[rid], far_end = far_beg + B.ann_len[rid];
                if (is_rev) {
                    const int64_t t = far_beg;
                    far_beg = (l_pac << 1) - far_end;
                    far_end = (l_pac << 1) - t;
                }
                rmax0 = rmax0 > far_beg ? rmax0 : far_beg;
                rmax1 = rmax1 < far_end ? rmax1 : far_end;
            }
            // seeds by (score, index) ascending; keys are distinct, so ranks give ks_introsort_64's order
            for (int i = lane; i < c.n; i += 32) {
                const uint64_t ki = (uint64_t)(uint32_t)cs[i].score << 32 | (uint32_t)i;
                int rank = 0;
                for (int j = 0; j < c.n; ++j)
                    rank += ((uint64_t)(uint32_t)cs[j].score << 32 | (uint32_t)j) < ki;
                srt[rank] = ki;
            }
            __syncwarp();
            for (int k = c.n - 1; k >= 0; --k) {
                const DevSeed s = cs[(uint32_t)srt[k]];
                // is the seed (almost) contained in a region of this read already? (bwamem.c:675-690)
                int hit = nav;
                for (int i0 = 0; i0 < nav && hit == nav; i0 += 32) {
                    const int i = i0 + lane;
                    bool ok = false;
                    if (i < nav) {
                        const bsb_reg_t p = av[i];
                        if (!(s.rbeg < p.rb || s.rbeg + s.len > p.re || s.qbeg < p.qb || s.qbeg + s.len > p.qe) &&
                            !(s.len - p.seedlen0 > .1 * l_query)) {
                            int qd = s.qbeg - p.qb;
                            int64_t rd = s.rbeg - p.rb;
                            int max_gap = cal_max_gap(opt, qd < rd ? qd : (int)rd);
                            int w = max_gap < p.w ? max_gap : p.w;
                            if (qd - rd < w && rd - qd < w) ok = true;
                            else {
                                qd = p.qe - (s.qbeg + s.len);
                                rd = p.re - (s.rbeg + s.len);
                                max_gap = cal_max_gap(opt, qd < rd ? qd : (int)rd);
                                w = max_gap < p.w ? max_gap : p.w;
                                ok = qd - rd < w && rd - qd < w;
                            }
                        }
                    }
                    const unsigned m = __ballot_sync(BSB_FULL_MASK, ok);
                    if (m) hit = i0 + __ffs(m) - 1;
                }
                if (hit < nav) {   // contained: extend only if an overlapping seed may lead elsewhere (bwamem.c:691-707)
                    int found = c.n;
                    for (int i0 = k + 1; i0 < c.n && found == c.n; i0 += 32) {
                        const int i = i0 + lane;
                        bool ok = false;
                        if (i < c.n && srt[i] != 0) {
                            const DevSeed t = cs[(uint32_t)srt[i]];
                            if (!(t.len < s.len * .95)) {
                                if (s.qbeg <= t.qbeg && s.qbeg + s.len - t.qbeg >= s.len >> 2 &&
                                    t.qbeg - s.qbeg != t.rbeg - s.rbeg)
                                    ok = true;
                                else if (t.qbeg <= s.qbeg && t.qbeg + t.len - s.qbeg >= s.len >> 2 &&
                                         s.qbeg - t.qbeg != s.rbeg - t.rbeg)
                                    ok = true;
                            }
                        }
                        const unsigned m = __ballot_sync(BSB_FULL_MASK, ok);
                        if (m) found = i0 + __ffs(m) - 1;
                    }
                    if (found == c.n) {
                        __syncwarp();
                        if (lane == 0) srt[k] = 0;
                        __syncwarp();
                        continue;
                    }
                }
                bsb_reg_t a;
                memset(&a, 0, sizeof a);
                int aw0 = opt.w, aw1 = opt.w;
                a.w = opt.w;
                a.score = a.truesc = -1;
                a.rid = c.rid;
                if (s.qbeg) {      // left extension (bwamem.c:715-748)
                    ReadRefAcc acc{query, s.qbeg - 1, -1, s.rbeg - 1, -1, B};
                    const int tlen = (int)(s.rbeg - rmax0);
                    KswResult x;
                    for (int i = 0; i < 2; ++i) {
                        const int prev = a.score;
                        aw0 = opt.w << i;
                        x = extend_any<MaxC>(P, s.qbeg, tlen, s.len * opt.a, aw0, opt.pen_clip5, acc, lane);
                        cells += x.cells;
                        a.score = x.score;
                        if (a.score == prev || x.max_off < (aw0 >> 1) + (aw0 >> 2)) break;
                    }
                    if (x.gscore <= 0 || x.gscore <= a.score - opt.pen_clip5) {
                        a.qb = s.qbeg - x.qle, a.rb = s.rbeg - x.tle;
                        a.truesc = a.score;
                    } else {
                        a.qb = 0, a.rb = s.rbeg - x.gtle;
                        a.truesc = x.gscore;
                    }
                } else a.score = a.truesc = s.len * opt.a, a.qb = 0, a.rb = s.rbeg;
                if (s.qbeg + s.len != l_query) {   // right extension (bwamem.c:750-775)
                    const int qe = s.qbeg + s.len, sc0 = a.score;
                    const int re = (int)(s.rbeg + s.len - rmax0);
                    ReadRefAcc acc{query, qe, 1, rmax0 + re, 1, B};
                    const int tlen = (int)(rmax1 - rmax0 - re);
                    KswResult x;
                    for (int i = 0; i < 2; ++i) {
                        const int prev = a.score;
                        aw1 = opt.w << i;
                        x = extend_any<MaxC>(P, l_query - qe, tlen, sc0, aw1, opt.pen_clip3, acc, lane);
                        cells += x.cells;
                        a.score = x.score;
                        if (a.score == prev || x.max_off < (aw1 >> 1) + (aw1 >> 2)) break;
                    }
                    if (x.gscore <= 0 || x.gscore <= a.score - opt.pen_clip3) {
                        a.qe = qe + x.qle, a.re = rmax0 + re + x.tle;
                        a.truesc += a.score - sc0;
                    } else {
                        a.qe = l_query, a.re = rmax0 + re + x.gtle;
                        a.truesc += x.gscore - sc0;
                    }
                } else a.qe = l_query, a.re = s.rbeg + s.len;
                int cov = 0;      // seedcov (bwamem.c:779-783)
                for (int i = lane; i < c.n; i += 32) {
                    const DevSeed t = cs[i];
                    if (t.qbeg >= a.qb && t.qbeg + t.len <= a.qe && t.rbeg >= a.rb && t.rbeg + t.len <= a.re) cov += t.len;
                }
                a.seedcov = __reduce_add_sync(BSB_FULL_MASK, cov);
                a.w = aw0 > aw1 ? aw0 : aw1;
                a.seedlen0 = s.len;
                a.frac_rep = c.frac_rep;
                if (lane == 0) av[nav] = a;
                ++nav;
                __syncwarp();
            }
        }
        if (lane == 0) {
            n_regs[r] = nav;
            if (read_cells) read_cells[r] = cells;
        }
    }
}

// ---------------------------------------------------------------- mem_flt_chained_seeds

// mem_flt_chained_seeds (bwamem.c:602-619) for the reads whose length makes it run
// (min_hsp[r] >= 0; the host evaluates the reference's double and float thresholds):
// each seed of each kept chain gets mem_seed_sw's score (bwamem.c:574-598) -- ksw_align2
// with KSW_XSTART over windows of 50 bases around the seed, on the GPU's ksw_align2 --
// and the chain keeps the seeds with no Smith-Waterman or a score of at least min_hsp,
// rescored.  seed_sw_window is mem_seed_sw up to its ksw_align2 call, with bns_fetch_seq's
// clip to the contig of the window's middle (bntseq.c:436-461); false: no SW, score -1.
constexpr int kSeedSwShortLen = 200, kSeedSwExt = 50;     // MEM_SHORT_LEN, MEM_SHORT_EXT

__device__ bool seed_sw_window(const DevBns &B, int l_query, const DevSeed &s, int &qb, int &qe, int64_t &rb,
                               int64_t &re)
{
    const int64_t l_pac = B.l_pac;
    if (s.len >= kSeedSwShortLen) return false;
    qb = s.qbeg, qe = s.qbeg + s.len;
    rb = s.rbeg, re = s.rbeg + s.len;
    const int64_t mid = (rb + re) >> 1;
    qb -= kSeedSwExt; qb = qb > 0 ? qb : 0;
    qe += kSeedSwExt; qe = qe < l_query ? qe : l_query;
    rb -= kSeedSwExt; rb = rb > 0 ? rb : 0;
    re += kSeedSwExt; re = re < l_pac << 1 ? re : l_pac << 1;
    if (rb < l_pac && l_pac < re) {
        if (mid < l_pac) re = l_pac;
        else rb = l_pac;
    }
    if (qe - qb >= kSeedSwShortLen || re - rb >= kSeedSwShortLen) return false;
    int is_rev;
    const int rid = pos2rid(B, depos(B, mid, is_rev));
    int64_t far_beg = B.ann_offset[rid], far_end = far_beg + B.ann_len[rid];
    if (is_rev) {
        const int64_t t = far_beg;
        far_beg = (l_pac << 1) - far_end;
        far_end = (l_pac << 1) - t;
    }
    rb = rb > far_beg ? rb : far_beg;
    re = re < far_end ? re : far_end;
    return true;
}

// Per read (thread per read): the Smith-Waterman jobs its seeds need and their bytes.
__global__ void seed_sw_count(DevBns B, int n_reads, const int *__restrict__ min_hsp,
                              const int64_t *__restrict__ read_off, const int64_t *__restrict__ seed_off,
                              const int64_t *__restrict__ row_off_of_seed, const DevSeed *__restrict__ seeds,
                              const DevChain *__restrict__ chains, const int *__restrict__ n_chains,
                              int *__restrict__ n_jobs, int64_t *__restrict__ n_bytes)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_reads; r += gridDim.x * blockDim.x) {
        int nj = 0;
        int64_t nb = 0;
        if (min_hsp[r] >= 0) {
            const int64_t R0 = row_off_of_seed[seed_off[r]];
            const int l_query = (int)(read_off[r + 1] - read_off[r]);
            for (int ci = 0; ci < n_chains[r]; ++ci) {
                const DevChain c = chains[R0 + ci];
                for (int i = 0; i < c.n; ++i) {
                    int qb, qe;
                    int64_t rb, re;
                    if (seed_sw_window(B, l_query, seeds[R0 + c.seed_off + i], qb, qe, rb, re))
                        ++nj, nb += (qe - qb) + (re - rb);
                }
            }
        }
        n_jobs[r] = nj;
        n_bytes[r] = nb;
    }
}

// The jobs (ksw_align2(qe-qb, query+qb, re-rb, rseq, ..., KSW_XSTART, 0)) and their bytes at
// each read's offsets, in chain and seed order.
__global__ void seed_sw_fill(DevBns B, int n_reads, const int *__restrict__ min_hsp,
                             const uint8_t *__restrict__ reads, const int64_t *__restrict__ read_off,
                             const int64_t *__restrict__ seed_off, const int64_t *__restrict__ row_off_of_seed,
                             const DevSeed *__restrict__ seeds, const DevChain *__restrict__ chains,
                             const int *__restrict__ n_chains, const int64_t *__restrict__ job_off,
                             const int64_t *__restrict__ byte_off, bsb_sw_job_t *__restrict__ jobs,
                             uint8_t *__restrict__ bytes)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_reads; r += gridDim.x * blockDim.x) {
        if (min_hsp[r] < 0) continue;
        const int64_t R0 = row_off_of_seed[seed_off[r]];
        const int l_query = (int)(read_off[r + 1] - read_off[r]);
        const uint8_t *q = reads + read_off[r];
        int64_t j = job_off[r], b = byte_off[r];
        for (int ci = 0; ci < n_chains[r]; ++ci) {
            const DevChain c = chains[R0 + ci];
            for (int i = 0; i < c.n; ++i) {
                int qb, qe;
                int64_t rb, re;
                if (!seed_sw_window(B, l_query, seeds[R0 + c.seed_off + i], qb, qe, rb, re)) continue;
                bsb_sw_job_t jb;
                jb.qoff = b, jb.qlen = qe - qb;
                for (int x = qb; x < qe; ++x) bytes[b++] = q[x];
                jb.toff = b, jb.tlen = (int32_t)(re - rb);
                for (int64_t x = rb; x < re; ++x) bytes[b++] = (uint8_t)text_base(B, x);
                jb.xtra = 0x80000;                                   // KSW_XSTART
                jb.pad_ = 0;
                jobs[j++] = jb;
            }
        }
    }
}

// The filter itself (bwamem.c:608-617): seeds keep their order, a seed without SW scores
// len * a, and chains shrink in place.
__global__ void seed_sw_apply(AlnOpt opt, DevBns B, int n_reads, const int *__restrict__ min_hsp,
                              const int64_t *__restrict__ read_off, const int64_t *__restrict__ seed_off,
                              const int64_t *__restrict__ row_off_of_seed, DevSeed *__restrict__ seeds,
                              DevChain *__restrict__ chains, const int *__restrict__ n_chains,
                              const int64_t *__restrict__ job_off, const int *__restrict__ score)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_reads; r += gridDim.x * blockDim.x) {
        const int mh = min_hsp[r];
        if (mh < 0) continue;
        const int64_t R0 = row_off_of_seed[seed_off[r]];
        const int l_query = (int)(read_off[r + 1] - read_off[r]);
        int64_t j = job_off[r];
        for (int ci = 0; ci < n_chains[r]; ++ci) {
            DevChain &c = chains[R0 + ci];
            DevSeed *cs = seeds + R0 + c.seed_off;
            int k = 0;
            for (int i = 0; i < c.n; ++i) {
                DevSeed sd = cs[i];
                int qb, qe;
                int64_t rb, re;
                const int sc = seed_sw_window(B, l_query, sd, qb, qe, rb, re) ? score[j++] : -1;
                if (sc < 0 || sc >= mh) {
                    sd.score = sc < 0 ? sd.len * opt.a : sc;
                    cs[k++] = sd;
                }
            }
            c.n = k;
        }
    }
}

// ---------------------------------------------------------------- learned read order

// Eight features per read for the learned extension-cost model (no reference counterpart:
// they only order the read queue of chain2aln_kernel), from the kept chains after the seed
// filter -- the inputs mem_chain2aln works from (bwamem.c:636-790):
//   f0 read length / 256          f1 log1p(kept chains) / 4     f2 log1p(their seeds) / 6
//   f3 best chain weight / length f4 mean seed offset / length  f5 chains on the reverse half
//   f6 C+G fraction of the read   f7 log2(1 + plain bound of the extension cells) / 24
// where the plain bound sums, over the seeds, the bases left and right of the seed times the
// band they are extended in (2w + 1).
__global__ void read_features_kernel(AlnOpt opt, DevBns B, int n_reads, const uint8_t *__restrict__ reads,
                                     const int64_t *__restrict__ read_off, const int64_t *__restrict__ seed_off,
                                     const int64_t *__restrict__ row_off_of_seed, const DevSeed *__restrict__ seeds,
                                     const DevChain *__restrict__ chains, const int *__restrict__ n_chains,
                                     float *__restrict__ feat)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_reads; r += gridDim.x * blockDim.x) {
        const int L = (int)(read_off[r + 1] - read_off[r]);
        const uint8_t *q = reads + read_off[r];
        const int64_t R0 = row_off_of_seed[seed_off[r]];
        int ns = 0, wmax = 0, nrev = 0, kept = 0, cg = 0;
        double qsum = 0., bound = 0.;
        for (int ci = 0; ci < n_chains[r]; ++ci) {
            const DevChain c = chains[R0 + ci];
            if (c.n == 0) continue;
            ++kept;
            wmax = c.w > wmax ? c.w : wmax;
            for (int i = 0; i < c.n; ++i) {
                const DevSeed sd = seeds[R0 + c.seed_off + i];
                ++ns;
                qsum += sd.qbeg;
                bound += (double)(L - sd.len) * (2 * opt.w + 1);
                nrev += sd.rbeg >= B.l_pac;
            }
        }
        for (int i = 0; i < L; ++i) cg += q[i] == 1 || q[i] == 2;
        float *f = feat + (int64_t)r * 8;
        const float l = L > 0 ? (float)L : 1.f;
        f[0] = L / 256.f;
        f[1] = log1pf((float)kept) / 4.f;
        f[2] = log1pf((float)ns) / 6.f;
        f[3] = wmax / l;
        f[4] = ns ? (float)(qsum / ns) / l : 0.f;
        f[5] = ns ? (float)nrev / ns : 0.f;
        f[6] = cg / l;
        f[7] = (float)(log2(1.0 + bound) / 24.0);
    }
}

// The learned order: reads by predicted cost, most expensive first, in 64 bins of half an
// octave of the predicted cells (key).
__device__ __forceinline__ int key_bin(int32_t key)
{
    if (key <= 0) return 63;
    const uint32_t k = (uint32_t)key;
    const int msb = 31 - __clz(k);
    const int half = 2 * msb + (msb > 0 ? (int)(k >> (msb - 1) & 1u) : 0);
    return 63 - (half < 63 ? half : 63);
}
__global__ void order_hist_key(const int32_t *__restrict__ key, int n_reads, int *__restrict__ cnt)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_reads; r += gridDim.x * blockDim.x)
        atomicAdd(&cnt[key_bin(key[r])], 1);
}
__global__ void order_scatter_key(const int32_t *__restrict__ key, int n_reads, const int *__restrict__ cnt,
                                  int *__restrict__ cur, int *__restrict__ order)
{
    __shared__ int off[64];
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int b = 0; b < 64; ++b) off[b] = acc, acc += cnt[b];
    }
    __syncthreads();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_reads; r += gridDim.x * blockDim.x) {
        const int b = key_bin(key[r]);
        order[off[b] + atomicAdd(&cur[b], 1)] = r;
    }
}

// The order chain2aln_kernel takes reads in: most chains first (reads are independent, so the
// order changes no result; it shortens the tail a few repeat-laden reads would otherwise set).
constexpr int kOrderBins = 64;

__device__ __forceinline__ int order_bin(int nc) { return kOrderBins - 1 - (nc < kOrderBins - 1 ? nc : kOrderBins - 1); }

__global__ void order_hist(const int *__restrict__ n_chains, int n_reads, int *__restrict__ cnt)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_reads; r += gridDim.x * blockDim.x)
        atomicAdd(&cnt[order_bin(n_chains[r])], 1);
}

__global__ void order_scatter(const int *__restrict__ n_chains, int n_reads, const int *__restrict__ cnt,
                              int *__restrict__ cur, int *__restrict__ order)
{
    __shared__ int off[kOrderBins];
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int b = 0; b < kOrderBins; ++b) off[b] = acc, acc += cnt[b];
    }
    __syncthreads();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_reads; r += gridDim.x * blockDim.x) {
        const int b = order_bin(n_chains[r]);
        order[off[b] + atomicAdd(&cur[b], 1)] = r;
    }
}

// One warp per read (reads hold a few regions each).
__global__ void compact_regs(const bsb_reg_t *__restrict__ regs, const int64_t *__restrict__ seed_off,
                             const int64_t *__restrict__ row_off_of_seed, int n_reads, const int *__restrict__ n_regs,
                             const int64_t *__restrict__ out_off, bsb_reg_t *__restrict__ out)
{
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (int r = blockIdx.x * wpb + (threadIdx.x >> 5); r < n_reads; r += gridDim.x * wpb) {
        const bsb_reg_t *src = regs + row_off_of_seed[seed_off[r]];
        for (int i = lane; i < n_regs[r]; i += 32) out[out_off[r] + i] = src[i];
    }
}

// ---------------------------------------------------------------- mem_sort_dedup_patch

struct RegReLt {                      // alnreg_slt2 (bwamem.c:395): by end
    const bsb_reg_t *r;
    __device__ bool operator()(int x, int y) const { return r[x].re < r[y].re; }
};

struct RegScoreLt {                   // alnreg_slt (bwamem.c:398): score down, then rb, qb up
    const bsb_reg_t *r;
    __device__ bool operator()(int x, int y) const
    {
        const bsb_reg_t &a = r[x], &b = r[y];
        return a.score > b.score || (a.score == b.score && (a.rb < b.rb || (a.rb == b.rb && a.qb < b.qb)));
    }
};

struct DedupOpt {
    int w, max_chain_gap;
    float mask_level_redun;
    GlobalPen pen;
    int8_t mat[25];
};

constexpr int kDedupWarps = 4;

struct DedupSmem {                    // one warp's global alignment of mem_patch_reg
    int32_t H[BSB_ALIGN_MAX_LEN + 1], E[BSB_ALIGN_MAX_LEN + 1];
    uint8_t q[BSB_ALIGN_MAX_LEN];
};

// Target base i of [rb, re) after bwa_gen_cigar2's flip (bwa.c:216-221): read backwards on the
// reverse strand.
struct PatchText {
    DevBns B;
    int64_t rb, re;
    bool rev;
    __device__ __forceinline__ int operator[](int i) const { return text_base(B, rev ? re - 1 - i : rb + i); }
};

// mem_patch_reg (bwamem.c:410-439) on the warp: every lane takes the same steps; the global
// alignment of its bwa_gen_cigar2 call (score only, bwa.c:211-244) runs on the whole warp.  The
// reference's double expressions are evaluated as written (no fused multiply-adds).
__device__ int patch_reg_warp(const DedupOpt &O, const int8_t *smat, const DevBns &B, const uint8_t *read,
                              const bsb_reg_t &a, const bsb_reg_t &b, int *w_out, DedupSmem &S, int lane)
{
    const int64_t l_pac = B.l_pac;
    if (a.rb < l_pac && b.rb >= l_pac) return 0;                       // different strands
    if (a.qb >= b.qb || a.qe >= b.qe || a.re >= b.re) return 0;       // not colinear
    int w = (int)((a.re - b.rb) - (a.qe - b.qb));
    w = w > 0 ? w : -w;
    double r = __dsub_rn(__ddiv_rn((double)(a.re - b.rb), (double)(b.re - a.rb)),
                         __ddiv_rn((double)(a.qe - b.qb), (double)(b.qe - a.qb)));
    r = r > 0. ? r : -r;
    if (a.re < b.rb || a.qe < b.qb) {
        if (w > O.w << 1 || r >= (double)0.05f) return 0;              // PATCH_MAX_R_BW
    } else if (w > O.w << 2 || r >= (double)(0.05f * 2)) return 0;
    w += a.w + b.w;
    w = w < O.w << 2 ? w : O.w << 2;
    // bwa_gen_cigar2(..., w, l_pac, pac, pac, b.qe - a.qb, query + a.qb, a.rb, b.re, &score, 0, ...)
    const int lq = b.qe - a.qb;
    const int64_t rb = a.rb, re = b.re;
    int score = 0;
    if (!(lq <= 0 || rb >= re || (rb < l_pac && re > l_pac)) && rb >= 0 && re <= l_pac << 1) {
        const bool rev = rb >= l_pac;
        const int rlen = (int)(re - rb);
        for (int j = lane; j < lq; j += 32) S.q[j] = read[rev ? b.qe - 1 - j : a.qb + j];
        __syncwarp();
        const PatchText T{B, rb, re, rev};
        if (lq == rlen && w == 0) {                                    // ungapped (bwa.c:222-230)
            int part = 0;
            for (int j = lane; j < lq; j += 32) part += smat[T[j] * 5 + S.q[j]];
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) part += __shfl_xor_sync(BSB_FULL_MASK, part, d);
            score = part;
        } else {                                                       // the band of bwa.c:232-240
            const int half = ((lq + 1) >> 1) * smat[0];
            const int max_ins = (int)__dadd_rn(__ddiv_rn((double)(half - O.pen.o_ins), (double)O.pen.e_ins), 1.);
            const int max_del = (int)__dadd_rn(__ddiv_rn((double)(half - O.pen.o_del), (double)O.pen.e_del), 1.);
            int max_gap = max_ins > max_del ? max_ins : max_del;
            max_gap = max_gap > 1 ? max_gap : 1;
            const int dl = rlen > lq ? rlen - lq : lq - rlen;
            int bw = (max_gap + dl + 1) >> 1;
            bw = bw < w ? bw : w;
            bw = bw > dl + 3 ? bw : dl + 3;
            score = global_rows_warp(O.pen, smat, S.q, lq, T, rlen, bw, 0, S.H, S.E, nullptr, lane);
        }
        __syncwarp();
    }
    const int sc2 = b.score + a.score;
    const int q_s = (int)__dadd_rn(__dmul_rn(__ddiv_rn((double)(b.qe - a.qb), (double)((b.qe - b.qb) + (a.qe - a.qb))),
                                             (double)sc2), .499);
    const int r_s = (int)__dadd_rn(__dmul_rn(__ddiv_rn((double)(b.re - a.rb), (double)((b.re - b.rb) + (a.re - a.rb))),
                                             (double)sc2), .499);
    if (__ddiv_rn((double)score, (double)(q_s > r_s ? q_s : r_s)) < (double)0.90f) return 0;   // PATCH_MIN_SC_RATIO
    *w_out = w;
    return score;
}

// mem_sort_dedup_patch (bwamem.c:441-493) per read, one warp per read.  in: the read's
// pre-dedup regions at reg_off[r]; a: scratch of the same size (the sorted copy that the scan
// edits); ix: index scratch; out: the kept regions at reg_off[r], n_out[r] of them.  Lane 0 runs
// the two ks_introsort orders; the redundancy and merge scan is taken by every lane in step
// (lane 0 writes), so that the warp can run a merge's global alignment.
__global__ void __launch_bounds__(kDedupWarps * 32)
dedup_kernel(DedupOpt O, DevBns B, int n_reads, const uint8_t *__restrict__ reads,
             const int64_t *__restrict__ read_off, const int64_t *__restrict__ reg_off,
             const bsb_reg_t *__restrict__ in, bsb_reg_t *a_all, int *ix_all, bsb_reg_t *__restrict__ out,
             int *__restrict__ n_out)
{
    __shared__ DedupSmem sm[kDedupWarps];
    __shared__ int8_t smat[25];
    if (threadIdx.x < 25) smat[threadIdx.x] = O.mat[threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, wb = threadIdx.x >> 5;
    for (int r = blockIdx.x * kDedupWarps + wb; r < n_reads; r += gridDim.x * kDedupWarps) {
        const int64_t o0 = reg_off[r];
        const int n = (int)(reg_off[r + 1] - o0);
        const bsb_reg_t *a_in = in + o0;
        bsb_reg_t *a = a_all + o0, *dst = out + o0;
        int *ix = ix_all + o0;
        if (n <= 1) {                                    // bwamem.c:444: returned as they are
            if (lane == 0) {
                if (n == 1) dst[0] = a_in[0];
                n_out[r] = n;
            }
            continue;
        }
        if (lane == 0) {                                 // sort by end (bwamem.c:445)
            int stk_l[64], stk_r[64], stk_d[64];
            for (int k = 0; k < n; ++k) ix[k] = k;
            KsSort<RegReLt>{ix, RegReLt{a_in}}.sort(n, stk_l, stk_r, stk_d);
        }
        __syncwarp();
        for (int k = lane; k < n; k += 32) {
            a[k] = a_in[ix[k]];
            a[k].n_comp = 1;
        }
        __syncwarp();
        const uint8_t *read = reads + read_off[r];
        for (int i = 1; i < n; ++i) {                    // bwamem.c:447-474
            bsb_reg_t p = a[i];
            if (p.rid != a[i - 1].rid || p.rb >= a[i - 1].re + O.max_chain_gap) continue;
            for (int j = i - 1; j >= 0 && p.rid == a[j].rid && p.rb < a[j].re + O.max_chain_gap; --j) {
                const bsb_reg_t q = a[j];
                if (q.qe == q.qb) continue;                      // a[j] has been excluded
                const int64_t or_ = q.re - p.rb;
                const int64_t oq = q.qb < p.qb ? q.qe - p.qb : p.qe - q.qb;
                const int64_t mr = q.re - q.rb < p.re - p.rb ? q.re - q.rb : p.re - p.rb;
                const int64_t mq = q.qe - q.qb < p.qe - p.qb ? q.qe - q.qb : p.qe - p.qb;
                // float, as the reference's float option times an int64
                if ((float)or_ > __fmul_rn(O.mask_level_redun, (float)mr) &&
                    (float)oq > __fmul_rn(O.mask_level_redun, (float)mq)) {
                    if (p.score < q.score) {
                        if (lane == 0) a[i].qe = p.qb;
                        __syncwarp();
                        break;
                    }
                    if (lane == 0) a[j].qe = q.qb;
                    __syncwarp();
                } else if (q.rb < p.rb) {
                    int w = 0;
                    const int score = patch_reg_warp(O, smat, B, read, q, p, &w, sm[wb], lane);
                    if (score > 0) {                             // merge q into p
                        if (lane == 0) {
                            p.n_comp += q.n_comp + 1;
                            p.seedcov = p.seedcov > q.seedcov ? p.seedcov : q.seedcov;
                            p.qb = q.qb, p.rb = q.rb;
                            p.truesc = p.score = score;
                            p.w = w;
                            a[i] = p;
                            a[j].qb = q.qe;
                        }
                        __syncwarp();
                        p = a[i];
                    }
                }
            }
        }
        __syncwarp();
        if (lane == 0) {                                 // bwamem.c:475-492
            int m = 0;
            for (int k = 0; k < n; ++k)
                if (a[k].qe > a[k].qb) ix[m++] = k;
            int cnt;
            if (m == 0) {                                // the reference then returns its first region
                dst[0] = a[0];
                cnt = 1;
            } else {
                int stk_l[64], stk_r[64], stk_d[64];
                KsSort<RegScoreLt>{ix, RegScoreLt{a}}.sort(m, stk_l, stk_r, stk_d);
                dst[0] = a[ix[0]];
                cnt = 1;
                for (int k = 1; k < m; ++k) {
                    const bsb_reg_t &x = a[ix[k]], &y = a[ix[k - 1]];
                    if (!(x.score == y.score && x.rb == y.rb && x.qb == y.qb)) dst[cnt++] = x;
                }
            }
            n_out[r] = cnt;
        }
        __syncwarp();
    }
}

__global__ void compact_kept(const bsb_reg_t *__restrict__ regs, const int64_t *__restrict__ in_off, int n_reads,
                             const int *__restrict__ n_kept, const int64_t *__restrict__ out_off,
                             bsb_reg_t *__restrict__ out)
{
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (int r = blockIdx.x * wpb + (threadIdx.x >> 5); r < n_reads; r += gridDim.x * wpb) {
        const bsb_reg_t *src = regs + in_off[r];
        for (int i = lane; i < n_kept[r]; i += 32) out[out_off[r] + i] = src[i];
    }
}

}  // namespace

// ---------------------------------------------------------------- host driver

struct AlignScratch {
    int *rcnt;                   // per seed interval: SA rows
    int64_t *roff;               // n_seeds + 1
    uint64_t *rows, *pos;
    ChainRec *chains;
    BtNode *nodes;
    int *row_chain, *iwork;
    DevSeed *cseeds;
    DevChain *cchains;
    uint64_t *srt;
    bsb_reg_t *regs;
    int *n_chains, *n_regs, *ctrl;
    int64_t *reg_off;
};

static size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

// dedup: also run mem_sort_dedup_patch per read (the regions mem_align1_core returns).
// The seed-level Smith-Waterman filter of the batch (mem_flt_chained_seeds) between chain_kernel
// and chain2aln_kernel, for the reads with h_min_hsp[r] >= 0: jobs and their bytes are built on
// the device, run through ksw_align2 on the GPU (bsb_align2_run, with staging of its own: d_in
// and d_out hold the batch meanwhile), and the scores go back to the chains on the device.
static int seed_sw_filter(bsb_ctx *ctx, const bsb_align_opt_t *o, const DevBns &B, int n_reads,
                          const int *h_min_hsp, const uint8_t *d_reads, const int64_t *d_read_off,
                          const int64_t *d_seed_off, const int64_t *roff, DevSeed *cseeds, DevChain *cchains,
                          const int *n_chains, const AlnOpt &ao)
{
    int rc;
    cudaStream_t st = ctx->stream;
    const size_t nr = (size_t)n_reads;
    const size_t head = al(4 * nr) + al(4 * nr) + al(8 * nr) + 2 * al(8 * (nr + 1));
    if ((rc = bsb_ensure(ctx, &ctx->flt_dev, &ctx->flt_dev_bytes, head + 256, "seed SW filter"))) return rc;
    char *D = (char *)ctx->flt_dev;
    int *d_mh = (int *)D, *d_nj = (int *)(D + al(4 * nr));
    int64_t *d_nb = (int64_t *)(D + 2 * al(4 * nr));
    int64_t *d_joff = (int64_t *)(D + 2 * al(4 * nr) + al(8 * nr)), *d_boff = d_joff + al(8 * (nr + 1)) / 8;
    const int grid = (int)std::min<int64_t>((n_reads + 127) / 128, (int64_t)ctx->n_sm * 8);
    std::vector<int> nj(nr);
    std::vector<int64_t> nbytes(nr), joff(nr + 1), boff(nr + 1);
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(d_mh, h_min_hsp, 4 * nr, cudaMemcpyHostToDevice, st), "H2D min_hsp")))
        return rc;
    seed_sw_count<<<grid, 128, 0, st>>>(B, n_reads, d_mh, d_read_off, d_seed_off, roff, cseeds, cchains, n_chains,
                                        d_nj, d_nb);
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(nj.data(), d_nj, 4 * nr, cudaMemcpyDeviceToHost, st), "D2H SW jobs")) ||
        (rc = bsb_cuda(ctx, cudaMemcpyAsync(nbytes.data(), d_nb, 8 * nr, cudaMemcpyDeviceToHost, st), "D2H SW bytes")) ||
        (rc = bsb_cuda(ctx, cudaStreamSynchronize(st), "seed SW count")))
        return rc;
    joff[0] = boff[0] = 0;
    for (size_t r = 0; r < nr; ++r) joff[r + 1] = joff[r] + nj[r], boff[r + 1] = boff[r] + nbytes[r];
    const int64_t NJ = joff[nr], NB = boff[nr];
    std::vector<int> score((size_t)NJ + 1);
    if (NJ > 0) {
        const size_t need = head + al(sizeof(bsb_sw_job_t) * (size_t)NJ) + al((size_t)NB) + al(4 * (size_t)NJ);
        if ((rc = bsb_ensure(ctx, &ctx->flt_dev, &ctx->flt_dev_bytes, need + 256, "seed SW filter"))) return rc;
        D = (char *)ctx->flt_dev;        // (re)allocated: recompute the views
        d_mh = (int *)D;
        d_joff = (int64_t *)(D + 2 * al(4 * nr) + al(8 * nr)), d_boff = d_joff + al(8 * (nr + 1)) / 8;
        bsb_sw_job_t *d_jobs = (bsb_sw_job_t *)(D + head);
        uint8_t *d_bytes = (uint8_t *)(D + head + al(sizeof(bsb_sw_job_t) * (size_t)NJ));
        if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(d_mh, h_min_hsp, 4 * nr, cudaMemcpyHostToDevice, st), "H2D min_hsp")) ||
            (rc = bsb_cuda(ctx, cudaMemcpyAsync(d_joff, joff.data(), 8 * (nr + 1), cudaMemcpyHostToDevice, st), "H2D")) ||
            (rc = bsb_cuda(ctx, cudaMemcpyAsync(d_boff, boff.data(), 8 * (nr + 1), cudaMemcpyHostToDevice, st), "H2D")))
            return rc;
        seed_sw_fill<<<grid, 128, 0, st>>>(B, n_reads, d_mh, d_reads, d_read_off, d_seed_off, roff, cseeds, cchains,
                                           n_chains, d_joff, d_boff, d_jobs, d_bytes);
        std::vector<bsb_sw_job_t> jobs((size_t)NJ);
        std::vector<uint8_t> bytes((size_t)NB + 1);
        std::vector<bsb_kswr_t> res((size_t)NJ);
        if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(jobs.data(), d_jobs, sizeof(bsb_sw_job_t) * NJ, cudaMemcpyDeviceToHost,
                                                st), "D2H SW jobs")) ||
            (rc = bsb_cuda(ctx, cudaMemcpyAsync(bytes.data(), d_bytes, NB, cudaMemcpyDeviceToHost, st), "D2H SW bytes")) ||
            (rc = bsb_cuda(ctx, cudaStreamSynchronize(st), "seed SW jobs")))
            return rc;
        bsb_ext_param_t p;
        memset(&p, 0, sizeof p);
        memcpy(p.mat, o->mat, 25);
        p.o_del = o->o_del, p.e_del = o->e_del, p.o_ins = o->o_ins, p.e_ins = o->e_ins, p.zdrop = o->zdrop;
        if ((rc = bsb_align2_run(ctx, &p, jobs.data(), NJ, bytes.data(), NB, res.data(), &ctx->flt_in,
                                 &ctx->flt_in_bytes, &ctx->flt_out, &ctx->flt_out_bytes)))
            return rc;
        for (int64_t i = 0; i < NJ; ++i) score[(size_t)i] = res[(size_t)i].score;
    }
    int *d_score = (int *)(D + head + al(sizeof(bsb_sw_job_t) * (size_t)NJ) + al((size_t)NB));
    if (NJ > 0 &&
        (rc = bsb_cuda(ctx, cudaMemcpyAsync(d_score, score.data(), 4 * (size_t)NJ, cudaMemcpyHostToDevice, st), "H2D")))
        return rc;
    seed_sw_apply<<<grid, 128, 0, st>>>(ao, B, n_reads, d_mh, d_read_off, d_seed_off, roff, cseeds, cchains, n_chains,
                                        d_joff, d_score);
    if ((rc = bsb_cuda(ctx, cudaGetLastError(), "seed SW filter"))) return rc;
    // the host vectors above must outlive the copies that read them
    return bsb_cuda(ctx, cudaStreamSynchronize(st), "seed SW filter");
}

static int bsb_align_regs_run(bsb_ctx *ctx, const bsb_align_opt_t *o, int n_reads, const uint8_t *d_reads,
                       const int64_t *d_read_off, const bsb_intv_t *d_seeds, const int64_t *d_seed_off,
                       int64_t n_seeds, int max_len, bool dedup, bsb_reg_t **d_regs_out, int64_t **d_reg_off_out,
                       int64_t *n_regs_total, const int *h_min_hsp)
{
    int rc;
    cudaStream_t st = ctx->stream;
    const int nb = ctx->n_sm * 4;
    // rows per seed interval and their offsets
    const int64_t scan_n = n_seeds > n_reads ? n_seeds : n_reads;
    size_t need = al(sizeof(int) * (n_seeds + 1)) + al(sizeof(int64_t) * (n_seeds + 1)) +
                  al(sizeof(int64_t) * scan_tmp_words(scan_n));
    if ((rc = bsb_ensure(ctx, &ctx->arena0, &ctx->arena0_bytes, need, "chain scratch (rows)"))) return rc;
    int *rcnt = (int *)ctx->arena0;
    int64_t *roff = (int64_t *)((char *)ctx->arena0 + al(sizeof(int) * (n_seeds + 1)));
    int64_t *scan_tmp = (int64_t *)((char *)roff + al(sizeof(int64_t) * (n_seeds + 1)));
    if (n_seeds > 0) {
        rows_count<<<nb, 256, 0, st>>>((const DevIntv *)d_seeds, n_seeds, o->max_occ, rcnt);
    }
    if ((rc = bsb_cuda(ctx, scan_i32_i64(rcnt, n_seeds, roff, scan_tmp, st), "row offsets"))) return rc;
    int64_t R = 0;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(&R, roff + n_seeds, 8, cudaMemcpyDeviceToHost, st), "row total"))) return rc;
    if ((rc = bsb_cuda(ctx, cudaStreamSynchronize(st), "row count"))) return rc;
    // per-row arrays (all sized by R)
    const size_t Rb = (size_t)(R > 0 ? R : 1);
    size_t off = 0;
    const size_t o_rows = off; off += al(8 * Rb);
    const size_t o_pos = off; off += al(8 * Rb);
    const size_t o_chains = off; off += al(sizeof(ChainRec) * Rb);
    const size_t o_nodes = off; off += al(sizeof(BtNode) * (Rb + 2));
    const size_t o_rowc = off; off += al(sizeof(int) * Rb);
    const size_t o_iwork = off; off += al(sizeof(int) * 3 * Rb);
    const size_t o_cseeds = off; off += al(sizeof(DevSeed) * Rb);
    const size_t o_cchains = off; off += al(sizeof(DevChain) * Rb);
    const size_t o_srt = off; off += al(8 * Rb);
    const size_t o_regs = off; off += al(sizeof(bsb_reg_t) * Rb);
    const size_t o_nch = off; off += al(sizeof(int) * (n_reads + 1));
    const size_t o_nreg = off; off += al(sizeof(int) * (n_reads + 1));
    const size_t o_ctrl = off; off += al(sizeof(int) * 4);
    const size_t o_regoff = off; off += al(sizeof(int64_t) * (n_reads + 1));
    const size_t o_out = off; off += al(sizeof(bsb_reg_t) * Rb);
    const size_t o_order = off; off += al(sizeof(int) * (n_reads + 1)) + al(sizeof(int) * 2 * kOrderBins);
    const size_t o_dtmp = off; off += dedup ? al(sizeof(bsb_reg_t) * Rb) : 0;
    const size_t o_dn = off; off += dedup ? al(sizeof(int) * (n_reads + 1)) : 0;
    const size_t o_doff = off; off += dedup ? al(sizeof(int64_t) * (n_reads + 1)) : 0;
    if ((rc = bsb_ensure(ctx, &ctx->arena1, &ctx->arena1_bytes, off, "chain scratch"))) return rc;
    char *A = (char *)ctx->arena1;
    uint64_t *rows = (uint64_t *)(A + o_rows), *pos = (uint64_t *)(A + o_pos);
    ChainRec *chains = (ChainRec *)(A + o_chains);
    BtNode *nodes = (BtNode *)(A + o_nodes);
    int *row_chain = (int *)(A + o_rowc), *iwork = (int *)(A + o_iwork);
    DevSeed *cseeds = (DevSeed *)(A + o_cseeds);
    DevChain *cchains = (DevChain *)(A + o_cchains);
    uint64_t *srt = (uint64_t *)(A + o_srt);
    bsb_reg_t *regs = (bsb_reg_t *)(A + o_regs), *regs_out = (bsb_reg_t *)(A + o_out);
    int *n_chains = (int *)(A + o_nch), *n_regs = (int *)(A + o_nreg), *ctrl = (int *)(A + o_ctrl);
    int64_t *reg_off = (int64_t *)(A + o_regoff);
    if ((rc = bsb_cuda(ctx, cudaMemsetAsync(ctrl, 0, sizeof(int) * 4, st), "ctrl"))) return rc;
    if (n_seeds > 0 && R > 0) {
        rows_fill<<<nb, 256, 0, st>>>((const DevIntv *)d_seeds, n_seeds, o->max_occ, roff, rows);
        cudaError_t e = bsb_sa_launch_ctx(ctx, rows, R, pos);
        if (e != cudaSuccess) return bsb_cuda(ctx, e, "SA rows");
    }
    if ((rc = bsb_cuda(ctx, cudaEventRecord(ctx->stage_ev[2], st), "stage mark"))) return rc;
    AlnOpt ao;
    ao.a = o->a; ao.o_del = o->o_del; ao.e_del = o->e_del; ao.o_ins = o->o_ins; ao.e_ins = o->e_ins;
    ao.w = o->w; ao.zdrop = o->zdrop; ao.pen_clip5 = o->pen_clip5; ao.pen_clip3 = o->pen_clip3;
    ao.min_seed_len = o->min_seed_len; ao.max_occ = o->max_occ; ao.max_chain_gap = o->max_chain_gap;
    ao.min_chain_weight = o->min_chain_weight; ao.max_chain_extend = o->max_chain_extend;
    ao.mask_level = o->mask_level; ao.drop_ratio = o->drop_ratio;
    DevBns B;
    B.ann_offset = (const int64_t *)ctx->idx_ann_off;
    B.ann_len = (const int32_t *)ctx->idx_ann_len;
    B.n_seqs = ctx->n_seqs;
    B.l_pac = ctx->l_pac;
    B.pac = (const uint8_t *)ctx->idx_pac;
    KswParams P;
    memcpy(P.mat, o->mat, 25);
    P.o_del = o->o_del; P.e_del = o->e_del; P.o_ins = o->o_ins; P.e_ins = o->e_ins; P.zdrop = o->zdrop;
    int mx = 0;
    for (int i = 0; i < 25; ++i) mx = mx > o->mat[i] ? mx : o->mat[i];
    P.mat_max = mx;
    P.pack16 = 0;
    chain_kernel<<<ctx->n_sm * 8, 128, 0, st>>>(ao, B, n_reads, d_read_off, (const DevIntv *)d_seeds, d_seed_off, roff,
                                                 pos, chains, nodes, row_chain, iwork, cseeds, cchains, n_chains, ctrl);
    if (h_min_hsp &&
        (rc = seed_sw_filter(ctx, o, B, n_reads, h_min_hsp, d_reads, d_read_off, d_seed_off, roff, cseeds, cchains,
                             n_chains, ao)))
        return rc;
    if ((rc = bsb_cuda(ctx, cudaEventRecord(ctx->stage_ev[3], st), "stage mark"))) return rc;
    int *order = (int *)(A + o_order);
    int *ocnt = (int *)(A + o_order + al(sizeof(int) * (n_reads + 1)));
    // per-read features / extension cells for the learned read order (kept for bsb_last_read_costs)
    float *d_feat = nullptr;
    int64_t *d_rcells = nullptr;
    int32_t *d_rkey = nullptr;
    const bool keyed = !ctx->order_keys.empty() && (int64_t)ctx->order_keys.size() == n_reads;
    if (!keyed) ctx->order_keys.clear();          // keys for another batch size are dropped
    const bool learned = ctx->read_model != nullptr && !keyed, logging = ctx->read_log != 0;
    if (learned || logging || keyed) {
        const size_t nr = (size_t)n_reads;
        if ((rc = bsb_ensure(ctx, &ctx->rc_buf, &ctx->rc_bytes, al(32 * nr) + al(8 * nr) + al(4 * nr) + 256,
                             "read costs")))
            return rc;
        d_feat = (float *)ctx->rc_buf;
        d_rcells = (int64_t *)((char *)ctx->rc_buf + al(32 * nr));
        d_rkey = (int32_t *)((char *)ctx->rc_buf + al(32 * nr) + al(8 * nr));
        const int fb = (int)std::min<int64_t>((n_reads + 127) / 128, (int64_t)ctx->n_sm * 8);
        if (learned || logging)
            read_features_kernel<<<fb, 128, 0, st>>>(ao, B, n_reads, d_reads, d_read_off, d_seed_off, roff, cseeds,
                                                     cchains, n_chains, d_feat);
        ctx->rc_n = logging ? n_reads : 0;
    }
    {
        const int ob = (int)((n_reads + 255) / 256) < ctx->n_sm * 4 ? (int)((n_reads + 255) / 256) : ctx->n_sm * 4;
        if ((rc = bsb_cuda(ctx, cudaMemsetAsync(ocnt, 0, sizeof(int) * 2 * kOrderBins, st), "read order"))) return rc;
        if (keyed) {         // the caller's keys, once (the copy is done before they are cleared)
            if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(d_rkey, ctx->order_keys.data(), sizeof(int32_t) * (size_t)n_reads,
                                                    cudaMemcpyHostToDevice, st), "read order keys")) ||
                (rc = bsb_cuda(ctx, cudaStreamSynchronize(st), "read order keys")))
                return rc;
            ctx->order_keys.clear();
            order_hist_key<<<ob, 256, 0, st>>>(d_rkey, n_reads, ocnt);
            order_scatter_key<<<ob, 256, 0, st>>>(d_rkey, n_reads, ocnt, ocnt + kOrderBins, order);
        } else if (learned) {   // predicted cells of every read, most expensive first
            if ((rc = bsb_mlp_forward(ctx, (const bsb_mlp_weights_t *)ctx->read_model, d_feat, n_reads, nullptr,
                                      d_rkey)))
                return rc;
            order_hist_key<<<ob, 256, 0, st>>>(d_rkey, n_reads, ocnt);
            order_scatter_key<<<ob, 256, 0, st>>>(d_rkey, n_reads, ocnt, ocnt + kOrderBins, order);
        } else {
            order_hist<<<ob, 256, 0, st>>>(n_chains, n_reads, ocnt);
            order_scatter<<<ob, 256, 0, st>>>(n_chains, n_reads, ocnt, ocnt + kOrderBins, order);
        }
    }
    int64_t *const rcells_out = logging ? d_rcells : nullptr;
    // every extension of these reads fits (max_len + 1) columns: the narrowest variant that holds them
    if (max_len <= 127)
        chain2aln_kernel<4><<<ctx->n_sm * 8, 128, 0, st>>>(ao, P, B, n_reads, d_reads, d_read_off, d_seed_off, roff,
                                                            cseeds, cchains, n_chains, srt, regs, n_regs, ctrl + 1, order, rcells_out);
    else if (max_len <= 159)
        chain2aln_kernel<5><<<ctx->n_sm * 8, 128, 0, st>>>(ao, P, B, n_reads, d_reads, d_read_off, d_seed_off, roff,
                                                            cseeds, cchains, n_chains, srt, regs, n_regs, ctrl + 1, order, rcells_out);
    else if (max_len <= 255)
        chain2aln_kernel<8><<<ctx->n_sm * 8, 128, 0, st>>>(ao, P, B, n_reads, d_reads, d_read_off, d_seed_off, roff,
                                                            cseeds, cchains, n_chains, srt, regs, n_regs, ctrl + 1, order, rcells_out);
    else if (max_len <= 511)
        chain2aln_kernel<16><<<ctx->n_sm * 4, 128, 0, st>>>(ao, P, B, n_reads, d_reads, d_read_off, d_seed_off, roff,
                                                             cseeds, cchains, n_chains, srt, regs, n_regs, ctrl + 1, order, rcells_out);
    else
        chain2aln_kernel<32><<<ctx->n_sm * 2, 128, 0, st>>>(ao, P, B, n_reads, d_reads, d_read_off, d_seed_off, roff,
                                                             cseeds, cchains, n_chains, srt, regs, n_regs, ctrl + 1, order, rcells_out);
    if ((rc = bsb_cuda(ctx, cudaEventRecord(ctx->stage_ev[4], st), "stage mark")) ||
        (rc = bsb_cuda(ctx, scan_i32_i64(n_regs, n_reads, reg_off, scan_tmp, st), "region offsets")))
        return rc;
    const int cgrid = (int)((n_reads + 3) / 4) < ctx->n_sm * 16 ? (int)((n_reads + 3) / 4) : ctx->n_sm * 16;
    compact_regs<<<cgrid, 128, 0, st>>>(regs, d_seed_off, roff, n_reads, n_regs, reg_off, regs_out);
    if (dedup) {
        // mem_sort_dedup_patch: regs_out (pre-dedup, at reg_off) -> regs (kept, at reg_off,
        // n_kept per read) -> regs_out again, compacted at the new offsets
        DedupOpt D;
        D.w = o->w, D.max_chain_gap = o->max_chain_gap, D.mask_level_redun = o->mask_level_redun;
        D.pen = GlobalPen{o->o_del, o->e_del, o->o_ins, o->e_ins};
        memcpy(D.mat, o->mat, 25);
        bsb_reg_t *dtmp = (bsb_reg_t *)(A + o_dtmp);
        int *n_kept = (int *)(A + o_dn);
        int64_t *kept_off = (int64_t *)(A + o_doff);
        const int db = (int)((n_reads + kDedupWarps - 1) / kDedupWarps);
        dedup_kernel<<<db < ctx->n_sm * 8 ? db : ctx->n_sm * 8, kDedupWarps * 32, 0, st>>>(
            D, B, n_reads, d_reads, d_read_off, reg_off, regs_out, dtmp, iwork, regs, n_kept);
        if ((rc = bsb_cuda(ctx, scan_i32_i64(n_kept, n_reads, kept_off, scan_tmp, st), "kept offsets"))) return rc;
        compact_kept<<<cgrid, 128, 0, st>>>(regs, reg_off, n_reads, n_kept, kept_off, regs_out);
        reg_off = kept_off;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return bsb_cuda(ctx, e, "chain/extension launch");
    if ((rc = bsb_cuda(ctx, cudaEventRecord(ctx->stage_ev[5], st), "stage mark")) ||
        (rc = bsb_cuda(ctx, cudaMemcpyAsync(n_regs_total, reg_off + n_reads, 8, cudaMemcpyDeviceToHost, st), "reg total")))
        return rc;
    if ((rc = bsb_cuda(ctx, cudaStreamSynchronize(st), "chain/extension"))) return rc;
    *d_regs_out = regs_out;
    *d_reg_off_out = reg_off;
    return 0;
}

static int align_batch(bsb_ctx *ctx, const bsb_align_opt_t *o, int32_t n_reads, const uint8_t *seqs,
                       const int64_t *offs, bsb_reg_t *regs, int64_t max_regs, int64_t *regs_off, bool dedup)
{
    if (!ctx) return BSB_EINVAL;
    if (!ctx->has_index || !ctx->idx_pac || !ctx->idx_ann_off)
        return bsb_fail(ctx, BSB_ENOINDEX, "no index with pac and contig table loaded");
    if (!o || !offs || n_reads < 0 || (n_reads > 0 && (!seqs || !regs || !regs_off)))
        return bsb_fail(ctx, BSB_EINVAL, "NULL argument");
    if (o->e_del < 1 || o->e_ins < 1 || o->o_del < 0 || o->o_ins < 0 || o->a < 1 || o->w < 0 || o->max_occ < 1 ||
        o->min_seed_len < 1 || o->max_chain_extend < 1)
        return bsb_fail(ctx, BSB_EINVAL, "unsupported options");
    if (n_reads == 0) {
        regs_off[0] = 0;
        return 0;
    }
    int max_len = 0;
    // mem_flt_chained_seeds (bwamem.c:602-606): per read length, its min_HSP_score when the
    // seed-level SW filter runs for that length, else -1 (the reference returns early)
    int hsp_of_len[BSB_ALIGN_MAX_LEN + 1];
    for (int l = 0; l <= BSB_ALIGN_MAX_LEN; ++l) {
        const double min_l = o->min_chain_weight ? 1.1f * o->min_chain_weight : 5.5f * log((double)l);
        hsp_of_len[l] = l > 0 && !(min_l > 0.05f * l) ? (int)(o->a * min_l + .499) : -1;
    }
    std::vector<int> min_hsp((size_t)n_reads);
    bool any_filter = false;
    for (int r = 0; r < n_reads; ++r) {
        const int64_t l = offs[r + 1] - offs[r];
        if (l < 0) return bsb_fail(ctx, BSB_EINVAL, "read %d: negative length", r);
        if (l > BSB_ALIGN_MAX_LEN) return bsb_fail(ctx, BSB_ETOOLONG, "read %d: length %lld > %d", r, (long long)l, BSB_ALIGN_MAX_LEN);
        min_hsp[(size_t)r] = hsp_of_len[l];
        any_filter |= hsp_of_len[l] >= 0;
        if (l > max_len) max_len = (int)l;
    }
    const int64_t total = offs[n_reads] - offs[0];
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    const size_t off_b = sizeof(int64_t) * ((size_t)n_reads + 1);
    const size_t seq_b = al((size_t)total);
    if ((rc = bsb_ensure(ctx, &ctx->d_in, &ctx->d_in_bytes, seq_b + 2 * al(off_b) + 256, "align input staging")))
        return rc;
    uint8_t *d_reads = (uint8_t *)ctx->d_in;
    int64_t *d_offs = (int64_t *)((char *)ctx->d_in + seq_b);
    int64_t *d_seed_off = (int64_t *)((char *)d_offs + al(off_b));
    std::vector<int64_t> rel(n_reads + 1);
    for (int r = 0; r <= n_reads; ++r) rel[r] = offs[r] - offs[0];
    ctx->stage_valid = false;
    cudaEvent_t *const sev = ctx->stage_ev;
    if ((rc = bsb_cuda(ctx, cudaEventRecord(sev[0], ctx->stream), "stage mark")) ||
        (rc = bsb_cuda(ctx, cudaMemcpyAsync(d_reads, seqs + offs[0], total, cudaMemcpyHostToDevice, ctx->stream), "H2D reads")))
        return rc;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(d_offs, rel.data(), off_b, cudaMemcpyHostToDevice, ctx->stream), "H2D offsets")))
        return rc;
    bsb_seed_opt_t so;
    so.min_seed_len = o->min_seed_len; so.split_factor = o->split_factor;
    so.split_width = o->split_width; so.max_mem_intv = o->max_mem_intv;
    // a read whose passes 1-2 overflow its seed slots: seeding again with twice the slots
    bsb_intv_t *d_seeds = nullptr;
    int64_t n_seeds = 0;
    for (int mult = 1;; mult *= 2) {
        const size_t seeds_b = al(seed_padded_entries(total, n_reads, mult) * sizeof(bsb_intv_t));
        if ((rc = bsb_ensure(ctx, &ctx->d_out, &ctx->d_out_bytes, seeds_b + 256, "align seed buffer"))) return rc;
        d_seeds = (bsb_intv_t *)ctx->d_out;
        if ((rc = bsb_seed_batch_device_m(ctx, &so, n_reads, d_reads, d_offs, total, max_len, d_seeds, d_seed_off,
                                          mult)) ||
            (rc = bsb_cuda(ctx, cudaEventRecord(sev[1], ctx->stream), "stage mark")))
            return rc;
        int ctrl[2] = {0, 0};
        if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(&n_seeds, d_seed_off + n_reads, 8, cudaMemcpyDeviceToHost, ctx->stream),
                           "seed total")) ||
            (rc = bsb_cuda(ctx, cudaMemcpyAsync(ctrl, ctx->seed_ctrl, sizeof ctrl, cudaMemcpyDeviceToHost, ctx->stream),
                           "seed ctrl")) ||
            (rc = bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "seeding")))
            return rc;
        if (!ctrl[1]) break;
        if (mult >= kSeedSlotMultMax)
            return bsb_fail(ctx, BSB_ETOOLONG, "read %d produced more seeds than %d times its buffer holds",
                            ctrl[1] - 1, mult);
        ++ctx->seed_regrown;
    }
    bsb_reg_t *d_regs = nullptr;
    int64_t *d_reg_off = nullptr, n_regs = 0;
    if ((rc = bsb_align_regs_run(ctx, o, n_reads, d_reads, d_offs, d_seeds, d_seed_off, n_seeds, max_len, dedup, &d_regs,
                                 &d_reg_off, &n_regs, any_filter ? min_hsp.data() : nullptr)))
        return rc;
    if ((rc = bsb_cuda(ctx, cudaMemcpyAsync(regs_off, d_reg_off, off_b, cudaMemcpyDeviceToHost, ctx->stream), "D2H offsets")))
        return rc;
    if (n_regs > max_regs) {
        // the offsets still go back: regs_off[n_reads] tells the caller the size to call again with
        if ((rc = bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "align batch"))) return rc;
        return bsb_fail(ctx, BSB_ECAPACITY, "%lld regions do not fit max_regs %lld", (long long)n_regs,
                        (long long)max_regs);
    }
    if (n_regs > 0 &&
        (rc = bsb_cuda(ctx, cudaMemcpyAsync(regs, d_regs, sizeof(bsb_reg_t) * n_regs, cudaMemcpyDeviceToHost, ctx->stream),
                       "D2H regions")))
        return rc;
    if ((rc = bsb_cuda(ctx, cudaEventRecord(sev[BSB_ALIGN_STAGES], ctx->stream), "stage mark")) ||
        (rc = bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "align batch")))
        return rc;
    ctx->stage_valid = true;
    return 0;
}

extern "C" int bsb_align_regs_batch(bsb_ctx *ctx, const bsb_align_opt_t *o, int32_t n_reads, const uint8_t *seqs,
                                    const int64_t *offs, bsb_reg_t *regs, int64_t max_regs, int64_t *regs_off)
{
    return align_batch(ctx, o, n_reads, seqs, offs, regs, max_regs, regs_off, false);
}

extern "C" int bsb_mem_align1_batch(bsb_ctx *ctx, const bsb_align_opt_t *o, int32_t n_reads, const uint8_t *seqs,
                                    const int64_t *offs, bsb_reg_t *regs, int64_t max_regs, int64_t *regs_off)
{
    if (!ctx) return BSB_EINVAL;
    if (o && !(o->mask_level_redun >= 0.f && o->mask_level_redun <= 1.f))
        return bsb_fail(ctx, BSB_EINVAL, "mask_level_redun must lie in [0, 1]");
    return align_batch(ctx, o, n_reads, seqs, offs, regs, max_regs, regs_off, true);
}

extern "C" int bsb_last_stage_ms(const bsb_ctx *ctx, float *ms, int n)
{
    if (!ctx || !ms || n < 0 || !ctx->stage_valid) return BSB_EINVAL;
    for (int k = 0; k < BSB_ALIGN_STAGES && k < n; ++k)
        if (cudaEventElapsedTime(&ms[k], ctx->stage_ev[k], ctx->stage_ev[k + 1]) != cudaSuccess) return BSB_ECUDA;
    return 0;
}

extern "C" int bsb_read_cost_log(bsb_ctx *ctx, int enable)
{
    if (!ctx) return BSB_EINVAL;
    ctx->read_log = enable != 0;
    ctx->rc_n = 0;
    return 0;
}

extern "C" int bsb_last_read_costs(bsb_ctx *ctx, int32_t n_reads, float *feat, int64_t *cells)
{
    if (!ctx) return BSB_EINVAL;
    if (!ctx->read_log || ctx->rc_n == 0) return bsb_fail(ctx, BSB_EINVAL, "no logged batch (bsb_read_cost_log)");
    if (n_reads != ctx->rc_n) return bsb_fail(ctx, BSB_EINVAL, "the logged batch has %d reads, not %d", ctx->rc_n, n_reads);
    int rc;
    if ((rc = bsb_cuda(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    const size_t nr = (size_t)n_reads;
    const char *b = (const char *)ctx->rc_buf;
    if (feat && (rc = bsb_cuda(ctx, cudaMemcpyAsync(feat, b, 32 * nr, cudaMemcpyDeviceToHost, ctx->stream), "D2H")))
        return rc;
    if (cells && (rc = bsb_cuda(ctx, cudaMemcpyAsync(cells, b + al(32 * nr), 8 * nr, cudaMemcpyDeviceToHost,
                                                     ctx->stream), "D2H")))
        return rc;
    return bsb_cuda(ctx, cudaStreamSynchronize(ctx->stream), "read costs");
}

extern "C" int bsb_set_read_cost_model(bsb_ctx *ctx, const bsb_mlp_weights_t *d_w)
{
    if (!ctx) return BSB_EINVAL;
    ctx->read_model = d_w;
    return 0;
}

extern "C" int bsb_set_read_order_keys(bsb_ctx *ctx, const int32_t *keys, int32_t n)
{
    if (!ctx) return BSB_EINVAL;
    if (n < 0 || (n > 0 && !keys)) return bsb_fail(ctx, BSB_EINVAL, "read order keys: NULL or negative count");
    ctx->order_keys.assign(keys, keys + (n > 0 ? n : 0));
    return 0;
}
