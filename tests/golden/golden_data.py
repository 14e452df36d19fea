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
        "L30": [1, 4, 6, 1, 6, 1, 100, 100, 30, 30, 19, 500, 10, 20, 10000]}


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
