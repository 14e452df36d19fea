// ksw_global.cuh -- the DP rows of ksw_global2 (bsbolt/External/BWA/ksw.c:504-582) on one warp,
// shared by bwa_gen_cigar2 (cigar.cu) and mem_patch_reg's score-only call (chain.cu).
#pragma once

#include <cstdint>

#include "bsb_internal.cuh"

constexpr int kNegInf = -0x40000000;        // MINUS_INF, ksw.c:490

struct GlobalPen {
    int o_del, e_del, o_ins, e_ins;
};

// The DP rows of ksw_global2 (ksw.c:519-582) on staged sequences (qs, ts after the strand
// flip), one warp: row i is processed 32 columns at a time, one column per lane.  At the
// start of cell j the reference holds eh[j] = {H(i-1, j-1), E(i, j)} and f = F(i, j); F
// depends only on the row's M values (F(i, j+1) = max(M(i, j) - oe_ins, F(i, j) - e_ins),
// F(i, beg) = -inf), so the lanes get it from a max-plus prefix scan -- max commutes with
// subtracting a constant, so the values are the reference's exactly -- and everything
// else in a cell is local.  H / E: qlen + 1 entries each (the reference's eh); Z: tlen
// rows of `stride` direction bytes, or NULL for the score alone (ksw_global2 without a
// CIGAR); ts[i]: target base i.  Returns the score on every lane.
template <class TS>
__device__ __forceinline__ int global_rows_warp(const GlobalPen &P, const int8_t *smat, const uint8_t *qs, int qlen,
                                                const TS &ts, int tlen, int w, int stride, int32_t *H, int32_t *E,
                                                uint8_t *Z, int lane)
{
    const int oe_del = P.o_del + P.e_del, oe_ins = P.o_ins + P.e_ins, e_ins = P.e_ins;
    for (int j = lane; j <= qlen; j += 32) {
        H[j] = j == 0 ? 0 : j <= w ? -(P.o_ins + e_ins * j) : kNegInf;
        E[j] = kNegInf;
    }
    __syncwarp();
    for (int i = 0; i < tlen; ++i) {
        const int8_t *srow = smat + ts[i] * 5;
        const int beg = i > w ? i - w : 0, end = i + w + 1 < qlen ? i + w + 1 : qlen;
        int32_t f_carry = kNegInf;                                        // F(i, j0)
        int32_t h_carry = beg == 0 ? -(P.o_del + P.e_del * (i + 1)) : kNegInf;   // H(i, j0 - 1)
        uint8_t *zrow = Z ? Z + (size_t)i * stride : nullptr;
        if (beg >= end && lane == 0) H[end] = h_carry, E[end] = kNegInf;     // an empty row (not reached: w > |tlen - qlen|)
        for (int j0 = beg; j0 < end; j0 += 32) {
            const int j = j0 + lane;
            const bool on = j < end;
            int32_t m = kNegInf, e = kNegInf;
            if (on) m = H[j] + srow[qs[j]], e = E[j];
            // out_L = F(i, j0+L+1) = max(m_L - oe_ins, out_{L-1} - e_ins), out_{-1} = f_carry;
            // with b_L = m_L - oe_ins + L*e_ins it is an inclusive max-scan shifted back
            int32_t sc = on ? m - oe_ins + lane * e_ins : INT32_MIN / 2;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int32_t v = __shfl_up_sync(BSB_FULL_MASK, sc, d);
                if (lane >= d) sc = sc > v ? sc : v;
            }
            const int32_t c0 = f_carry - e_ins;                          // out_{-1}, normalised at L = -1
            const int32_t out = (sc > c0 ? sc : c0) - lane * e_ins;      // F(i, j + 1)
            int32_t f = __shfl_up_sync(BSB_FULL_MASK, out, 1);          // F(i, j)
            if (lane == 0) f = f_carry;
            int32_t h, t;
            uint32_t dir;
            if (m >= e) h = m, dir = 0;
            else h = e, dir = 1;
            if (h < f) h = f, dir = 2;
            t = m - oe_del;
            e -= P.e_del;
            if (e > t) dir |= 1 << 2;
            else e = t;
            t = m - oe_ins;
            if (f - e_ins > t) dir |= 2 << 4;
            int32_t hprev = __shfl_up_sync(BSB_FULL_MASK, h, 1);        // H(i, j - 1)
            if (lane == 0) hprev = h_carry;
            if (on) {
                H[j] = hprev;
                E[j] = e;
                if (zrow) zrow[j - beg] = (uint8_t)dir;
                if (j == end - 1) H[end] = h, E[end] = kNegInf;
            }
            f_carry = __shfl_sync(BSB_FULL_MASK, out, 31);
            h_carry = __shfl_sync(BSB_FULL_MASK, h, 31);
        }
        __syncwarp();
    }
    return H[qlen];
}

