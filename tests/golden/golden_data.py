"""Seeded inputs shared by the golden-fixture generator and the tests.

The test reference and read set are regenerated from seeds wherever they are
needed (here, and on machines without the reference sources), so only the
reference's outputs have to be stored as fixtures.
"""
import numpy as np

import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
from bsbolt_gb300 import synth  # noqa: E402

GENOME = dict(n_contigs=3, contig_len=120_000, seed=20261203)


def golden_genome():
    """The seeded test reference: 3 x 120 kb at GC 41 % with thinned CpG, plus a
    5 kb duplicated block (as in the reference's own BSB_test.fa), a tandem
    repeat, and an N run, so seeds hit repeats and the index has holes."""
    contigs = synth.bs_genome(**GENOME)
    c0 = contigs[0][1]
    c2 = contigs[2][1]
    c2[10_000:15_000] = c0[50_000:55_000]            # duplicated block
    unit = c0[70_000:70_037].copy()
    c2[40_000:40_000 + 37 * 20] = np.tile(unit, 20)  # tandem repeat
    contigs[1][1][60_000:60_050] = 4                 # N run
    return contigs


# a, b, o_del, e_del, o_ins, e_ins, w, zdrop, pen_clip5, pen_clip3,
# min_seed_len, max_occ, split_width, max_mem_intv, max_chain_gap
OPTS = {"L5": [1, 4, 6, 1, 6, 1, 100, 100, 5, 5, 19, 500, 10, 20, 10000],
        "L30": [1, 4, 6, 1, 6, 1, 100, 100, 30, 30, 19, 500, 10, 20, 10000],
        # a narrow band: indels of a few bases split chains, so mem_sort_dedup_patch merges
        # colinear regions (mem_patch_reg) as well as dropping redundant ones
        "W5": [1, 4, 6, 1, 6, 1, 5, 100, 5, 5, 19, 500, 10, 20, 10000]}


def golden_reads(n_pairs=700, seed=20261203 + 7):
    contigs = golden_genome()
    contigs = [(n, np.where(c > 3, 0, c).astype(np.uint8)) for n, c in contigs]
    r1, r2 = synth.bs_reads_pe(contigs, n_pairs, read_len=100, seed=seed)
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    reads = []
    for a, b in zip(r1, r2):
        reads.append(synth.bs_convert(a, g2a=False))
        reads.append(synth.bs_convert(b, g2a=True))
    # a few ragged / short / N-rich reads
    reads.append(np.zeros(0, np.uint8))
    reads.append(rng.integers(0, 4, 12).astype(np.uint8))
    reads.append(np.concatenate([reads[0][:50], np.full(5, 4, np.uint8), reads[0][50:]]))
    reads.append(rng.integers(0, 5, 250).astype(np.uint8))
    reads.append(np.tile(np.array([0, 3], np.uint8), 75))
    return reads




def golden_reads_indel(n=400, seed=20261203 + 8):
    """Reads of 150-300 bases from the golden genome (both strands, converted), each with
    one or two indels of 6-14 bases, plus copies that repeat a 20-60 base stretch: with
    the W5 band their seeds fall into several chains, and their regions into the merge
    and redundancy cases of mem_sort_dedup_patch."""
    contigs = golden_genome()
    contigs = [(nm, np.where(c > 3, 0, c).astype(np.uint8)) for nm, c in contigs]
    rng = np.random.Generator(np.random.PCG64(seed))
    reads = []
    for k in range(n):
        c = contigs[int(rng.integers(0, len(contigs)))][1]
        L = int(rng.integers(150, 301))
        at = int(rng.integers(0, len(c) - L - 100))
        frag = c[at:at + L + 60].copy()
        for _ in range(int(rng.choice([1, 1, 2]))):
            pos = int(rng.integers(40, L - 40))
            ln = int(rng.integers(6, 15))
            if rng.random() < 0.5:
                frag = np.concatenate([frag[:pos], frag[pos + ln:]])
            else:
                frag = np.concatenate([frag[:pos], rng.integers(0, 4, ln).astype(np.uint8), frag[pos:]])
        if k % 4 == 3:                                  # a repeated stretch (tandem duplication)
            pos, ln = int(rng.integers(40, L - 80)), int(rng.integers(20, 61))
            frag = np.concatenate([frag[:pos + ln], frag[pos:pos + ln], frag[pos + ln:]])
        r = frag[:L]
        if k % 2:
            r = (3 - r[::-1]).astype(np.uint8)
        reads.append(synth.bs_convert(r, g2a=bool(k % 3 == 0)))
    return reads


# ------------------------------------------------------------ repeat stress

GENOME_REP = dict(seed=20261203 + 99)


def golden_genome_rep():
    """A 2 x 150 kb reference where 60 copies of a 300 bp element (0-3 %
    divergence) and 40 exact copies of a 120 bp element are scattered, so
    reads hit dozens of loci: many chains per read (B-tree splits), chains
    of equal weight (sort ties) and heavy SA sampling (max_occ)."""
    rng = np.random.Generator(np.random.PCG64(GENOME_REP["seed"]))
    contigs = synth.bs_genome(2, 150_000, seed=GENOME_REP["seed"])
    elem = contigs[0][1][1000:1300].copy()
    small = contigs[1][1][2000:2120].copy()
    for k in range(60):
        c = contigs[k % 2][1]
        at = int(rng.integers(5000, len(c) - 400))
        e = elem.copy()
        mut = rng.random(len(e)) < (k % 4) * 0.01
        e[mut] = rng.integers(0, 4, int(mut.sum()))
        c[at:at + len(e)] = e
    for k in range(40):
        c = contigs[k % 2][1]
        at = int(rng.integers(5000, len(c) - 200))
        c[at:at + len(small)] = small
    return contigs


def golden_reads_rep(n=400, seed=20261203 + 100):
    rng = np.random.Generator(np.random.PCG64(seed))
    contigs = golden_genome_rep()
    elem = contigs[0][1][1000:1300]
    reads = []
    for k in range(n):
        kind = k % 4
        c = contigs[int(rng.integers(0, 2))][1]
        if kind == 0:        # a read inside a repeat element
            st = int(rng.integers(0, 200))
            r = elem[st:st + 100].copy()
        elif kind == 1:      # a genomic read that crosses into repeats
            L = int(rng.integers(100, 251))
            st = int(rng.integers(0, len(c) - L))
            r = c[st:st + L].copy()
        elif kind == 2:      # the same 40-mer twice, 150 bp apart: chains with equal keys
            st = int(rng.integers(0, len(c) - 60))
            u = c[st:st + 40].copy()
            r = np.concatenate([u, rng.integers(0, 4, 110), u, rng.integers(0, 4, 60)]).astype(np.uint8)
        else:                # a strand-flipped repeat read with errors
            st = int(rng.integers(0, 150))
            r = (3 - elem[st:st + 150][::-1]).astype(np.uint8)
        e = rng.random(len(r)) < 0.01
        r[e] = rng.integers(0, 4, int(e.sum()))
        reads.append(synth.bs_convert(r.astype(np.uint8), g2a=bool(k & 1)))
    return reads


# ------------------------------------------------------- CIGAR / MD / XB jobs

CIGAR_JOB_DTYPE = np.dtype([("rb", "<i8"), ("re", "<i8"), ("qoff", "<i8"), ("ooff", "<i8"),
                            ("l_query", "<i4"), ("w", "<i4")])


def pac_codes(pac, lo, hi):
    """Forward-strand codes of positions [lo, hi) of a 2-bit pac (_get_pac, bntseq.h:79)."""
    k = np.arange(lo, hi, dtype=np.int64)
    return ((pac[k >> 2] >> ((~k & 3) << 1)) & 3).astype(np.uint8)


def doubled_seq(pac, l_pac, beg, end):
    """Bases of [beg, end) of the doubled sequence (one strand, no clamping): bns_get_seq."""
    if beg >= l_pac:
        return (3 - pac_codes(pac, 2 * l_pac - end, 2 * l_pac - beg)[::-1]).astype(np.uint8)
    return pac_codes(pac, beg, end)


def _edit(rng, seqs, sub, n_indel):
    """The same substitutions and indels applied to parallel sequences."""
    seqs = [s.copy() for s in seqs]
    L = len(seqs[0])
    e = np.nonzero(rng.random(L) < sub)[0]
    for s in seqs:
        s[e] = (s[e] + 1 + (e % 3)) % 4
    for _ in range(n_indel):
        at = int(rng.integers(1, max(2, len(seqs[0]) - 1)))
        ln = int(rng.integers(1, 6))
        if rng.random() < 0.5:
            ins = rng.integers(0, 4, ln).astype(np.uint8)
            seqs = [np.concatenate([s[:at], ins, s[at:]]) for s in seqs]
        else:
            seqs = [np.concatenate([s[:at], s[at + ln:]]) for s in seqs]
    return seqs


def golden_cigar_jobs(pac, opac, l_pac, crick_l, n_random=500, seed=20261203 + 11):
    """bwa_gen_cigar2 jobs against a bisulfite index (pac = converted, opac = original
    bases): reads drawn from both strands of Watson and Crick contigs with mismatches,
    indels and partial methylation, region starts inside the read (mem_reg2aln hands the
    whole original read with query + qb, bwamem.c:1228), the bands mem_reg2aln tries,
    the ungapped w = 0 path, unrelated sequences, and the rejected / no-MD corner cases.
    Returns (jobs[CIGAR_JOB_DTYPE], qbuf, obuf, tags) -- tags name each job's kind."""
    rng = np.random.Generator(np.random.PCG64(seed))
    jobs, qparts, oparts, tags = [], [], [], []
    qn = on = 0

    def add(rb, re, q, oq, w, tag, qb=0):
        nonlocal qn, on
        q = np.asarray(q, np.uint8)
        oq = np.asarray(oq, np.uint8)
        jobs.append((rb, re, qn + qb, on, len(q) - qb, w))
        qparts.append(q)
        oparts.append(oq)
        qn += len(q)
        on += len(oq)
        tags.append(tag)

    def methylate(oref, frac):
        oq = oref.copy()
        for c, t in ((1, 3), (2, 0)):
            m = (oq == c) & (rng.random(len(oq)) > frac)
            oq[m] = t
        return oq

    widths = np.array([0, 1, 2, 5, 10, 20, 40, 100, 200, 400])
    for i in range(n_random):
        L = int(rng.integers(20, 251))
        rev = bool(rng.random() < 0.5)
        base = int(rng.integers(3, l_pac - L - 10))
        rb = base + (l_pac if rev else 0)
        ref = doubled_seq(pac, l_pac, rb, rb + L)
        oref = doubled_seq(opac, l_pac, rb, rb + L)
        oq0 = methylate(oref, rng.random())
        n_indel = int(rng.choice([0, 0, 0, 1, 2, 3]))
        q, oq = _edit(rng, [ref, oq0], float(rng.choice([0.0, 0.01, 0.03, 0.08])), n_indel)
        if rng.random() < 0.1:
            q[rng.random(len(q)) < 0.05] = 4                    # N in the read
        re = rb + L + int(rng.integers(-3, 4)) * (i % 3 == 0)
        w = int(rng.choice(widths))
        if len(q) != re - rb and w == 0:
            w = int(rng.choice(widths[1:]))
        qb = int(rng.integers(0, 12)) if i % 4 == 0 else 0      # region starting inside the read
        if qb:
            pre = rng.integers(0, 4, qb).astype(np.uint8)
            q = np.concatenate([pre, q])
            oq = np.concatenate([pre, oq])
        add(rb, re, q, oq, w, "random", qb)
    for rev in (0, 1):                                          # ungapped path (bwa.c:222-230)
        for L in (30, 100, 151):
            rb = int(rng.integers(10, l_pac - 300)) + rev * l_pac
            ref = doubled_seq(pac, l_pac, rb, rb + L)
            oq = methylate(doubled_seq(opac, l_pac, rb, rb + L), 0.5)
            q, oq = _edit(rng, [ref, oq], 0.02, 0)
            add(rb, rb + L, q, oq, 0, "ungapped")
    for w in (10, 100, 400):                                    # unrelated sequences: long CIGARs
        for L in (40, 120, 250):
            rb = int(rng.integers(10, 2 * l_pac - 400))
            if rb < l_pac < rb + L + 5:
                rb = l_pac + 10
            q = rng.integers(0, 4, L).astype(np.uint8)
            add(rb, rb + L + 5, q, rng.integers(0, 4, L), w, "unrelated")
    # corner cases of the interval (bwa.c:211-215, 264-266)
    q = doubled_seq(pac, l_pac, 1000, 1100)
    oq = doubled_seq(opac, l_pac, 1000, 1100)
    add(1000, 1100, q[:0], oq[:0], 10, "reject_empty_query")
    add(1000, 1000, q, oq, 10, "reject_empty_ref")
    add(1100, 1000, q, oq, 10, "reject_reversed")
    add(l_pac - 50, l_pac + 50, q, oq, 10, "reject_bridging")
    for rb, re, tag in ((l_pac - 100, l_pac, "no_md_forward_end"), (l_pac - 101, l_pac - 1, "no_md_forward_end1"),
                        (l_pac, l_pac + 100, "no_md_reverse_start"), (l_pac + 1, l_pac + 101, "no_md_reverse_start1"),
                        (l_pac + 2, l_pac + 102, "reverse_first_context"), (l_pac - 102, l_pac - 2, "forward_last_context"),
                        (2, 102, "forward_first_context"), (2 * l_pac - 102, 2 * l_pac - 2, "reverse_last_context"),
                        (crick_l - 50, crick_l + 50, "crick_boundary"), (crick_l, crick_l + 100, "crick_start"),
                        (crick_l + l_pac - 50, crick_l + l_pac + 50, "crick_boundary_rev"),
                        (crick_l + l_pac, crick_l + l_pac + 100, "crick_start_rev")):
        ref = doubled_seq(pac, l_pac, rb, re)
        oref = doubled_seq(opac, l_pac, rb, re)
        q, oq = _edit(rng, [ref, methylate(oref, 0.4)], 0.02, 1)
        add(rb, re, q, oq, 20, tag)
    for rb, re, tag in ((0, 100, "clipped_start"), (1, 101, "clipped_start1"),
                        (2 * l_pac - 100, 2 * l_pac, "clipped_end"), (2 * l_pac - 101, 2 * l_pac - 1, "clipped_end1")):
        ref = doubled_seq(pac, l_pac, rb, re)
        oref = doubled_seq(opac, l_pac, rb, re)
        add(rb, re, ref, oref, 20, tag)
    add(5000, 5100, doubled_seq(pac, l_pac, 5000, 5100), doubled_seq(opac, l_pac, 5000, 5100), 0, "perfect_w0")
    jobs = np.array(jobs, CIGAR_JOB_DTYPE)
    return jobs, np.concatenate(qparts), np.concatenate(oparts), np.array(tags)


# ------------------------------------------------- mate-rescue Smith-Waterman jobs

SW_JOB_DTYPE = np.dtype([("qoff", "<i8"), ("toff", "<i8"), ("qlen", "<i4"), ("tlen", "<i4"), ("xtra", "<i4"),
                         ("pad", "<i4")])
KSW_XBYTE, KSW_XSTOP, KSW_XSUBO, KSW_XSTART = 0x10000, 0x20000, 0x40000, 0x80000


def golden_sw_jobs(a=1, n=1200, seed=20261203 + 21):
    """ksw_align2 jobs shaped like mem_matesw's (bwamem_pair.c:135-160): a mate read of 30-250
    bases against a reference window of a few hundred bases that holds a mutated copy of it
    (or does not), with the flags mem_matesw passes -- XSUBO | XSTART | min_seed_len*a, plus
    XBYTE when qlen*a < 250 -- and the other flag combinations of the interface: none, XSTART
    alone, XSTOP, XSUBO thresholds, byte lanes on long queries (saturation, without XSTART:
    the reference's start pass is undefined there), tiny queries and targets.
    Returns (jobs[SW_JOB_DTYPE], seq, tags)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    jobs, parts, tags = [], [], []
    off = 0

    def add(q, t, xtra, tag):
        nonlocal off
        q = np.asarray(q, np.uint8)
        t = np.asarray(t, np.uint8)
        jobs.append((off, off + len(q), len(q), len(t), int(xtra), 0))
        parts.extend([q, t])
        off += len(q) + len(t)
        tags.append(tag)

    for k in range(n):
        L = int(rng.integers(30, 251))
        q = rng.integers(0, 4, L).astype(np.uint8)
        q[rng.random(L) < 0.01] = 4
        wl = int(rng.integers(L + 20, L + 700))
        t = rng.integers(0, 4, wl).astype(np.uint8)
        kind = k % 5
        if kind < 4:                                       # the mate inside the window
            m = q.copy()
            sub = rng.random(L) < float(rng.choice([0.0, 0.01, 0.05, 0.15]))
            m[sub] = rng.integers(0, 4, int(sub.sum()))
            for _ in range(int(rng.choice([0, 0, 1, 2]))):
                at = int(rng.integers(1, len(m) - 1))
                ln = int(rng.integers(1, 6))
                m = np.concatenate([m[:at], rng.integers(0, 4, ln).astype(np.uint8), m[at:]]) if rng.random() < .5 \
                    else np.concatenate([m[:at], m[at + ln:]])
            m = m[: wl]
            at = int(rng.integers(0, wl - len(m) + 1))
            t[at:at + len(m)] = m
            if kind == 3:                                  # a second, weaker copy: a suboptimal hit
                at2 = int(rng.integers(0, max(1, wl - len(m) + 1)))
                if abs(at2 - at) > L:
                    m2 = m.copy()
                    s2 = rng.random(len(m2)) < 0.2
                    m2[s2] = rng.integers(0, 4, int(s2.sum()))
                    t[at2:at2 + len(m2)] = m2[: wl - at2]
        flags = [KSW_XSUBO | KSW_XSTART | (KSW_XBYTE if L * a < 250 else 0) | (19 * a),   # mem_matesw
                 0, KSW_XSTART, KSW_XSTART | (KSW_XBYTE if L * a < 250 else 0),
                 KSW_XSUBO | int(rng.integers(1, 60)), KSW_XSTOP | int(rng.integers(10, 120))]
        add(q, t, flags[k % len(flags)], ["matesw", "plain", "start", "start-byte", "subo", "stop"][k % len(flags)])
    for L in (1, 2, 3, 7, 15, 16, 17, 31, 32, 33, 48):     # lane and segment boundaries
        q = rng.integers(0, 4, L).astype(np.uint8)
        t = np.concatenate([rng.integers(0, 4, 20), q, rng.integers(0, 4, 20)]).astype(np.uint8)
        for xtra in (KSW_XSTART, KSW_XSTART | KSW_XBYTE, KSW_XSUBO | KSW_XSTART | 5):
            add(q, t, xtra, "short")
    add(rng.integers(0, 4, 40), np.zeros(0, np.uint8), KSW_XSTART, "empty-target")
    add(rng.integers(0, 4, 40), rng.integers(0, 4, 1), KSW_XSTART, "one-row")
    for L in (300, 400, 600):                               # byte lanes that saturate (no start pass)
        q = rng.integers(0, 4, L).astype(np.uint8)
        t = np.concatenate([rng.integers(0, 4, 50), q, rng.integers(0, 4, 50)]).astype(np.uint8)
        add(q, t, KSW_XBYTE | KSW_XSUBO | 19, "byte-saturated")
        add(q, t, KSW_XSTART, "long-i16")
    return np.array(jobs, SW_JOB_DTYPE), np.concatenate(parts), np.array(tags)
