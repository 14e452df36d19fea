"""The chaining / chain-filter / mem_chain2aln / mem_sort_dedup_patch oracle against
the reference (CPU only).

Fixtures (tests/golden/reads*_*.npz) hold, per read, the reference's chains
straight out of mem_chain (tree order), after mem_chain_flt, the pre-dedup
regions of mem_chain2aln and the regions after mem_sort_dedup_patch.  The
repeat-stress set has reads with up to 125 chains (B-tree splits), equal chain
keys and tied chain weights; the indel set (band 5) has regions that
mem_patch_reg merges and regions dropped as redundant.
"""
import os
import sys

import numpy as np
import pytest

import oracle
from bsbolt_gb300 import index, synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import golden_data  # noqa: E402

CASES = [("reads_L5.npz", golden_data.golden_genome), ("reads_L30.npz", golden_data.golden_genome),
         ("reads_rep_L5.npz", golden_data.golden_genome_rep), ("reads_indel_W5.npz", golden_data.golden_genome)]
_IDX = {}


def index_for(genome, tmp_path_factory):
    if genome not in _IDX:
        d = tmp_path_factory.mktemp("cidx")
        fa = str(d / "ref.fa")
        synth.write_fasta(fa, genome())
        index.build_index(fa, str(d / "ref"))
        _IDX[genome] = index.BwaIndex(str(d / "ref"))
    return _IDX[genome]


def check_against_golden(r, g):
    c0, gc0 = r["chain0"], g["chain0_rows"]
    assert np.array_equal(r["chain0_off"], g["chain0_off"])
    for i, f in [(0, "n"), (1, "rid"), (5, "pos")]:
        assert np.array_equal(c0[f], gc0[:, i]), f"chain0.{f}"
    assert np.array_equal(c0["frac_rep"].view(np.int32), gc0[:, 4].astype(np.int32))
    s0, gs = r["seeds0"], g["chain0_seeds"]
    for i, f in enumerate(["rbeg", "qbeg", "len", "score"]):
        assert np.array_equal(s0[f], gs[:, i]), f"seed.{f}"
    c1, gc1 = r["chain1"], g["chain1_rows"]
    assert np.array_equal(r["chain1_off"], g["chain1_off"])
    for i, f in [(0, "n"), (1, "rid"), (2, "kept"), (3, "w"), (4, "first"), (5, "pos")]:
        assert np.array_equal(c1[f], gc1[:, i]), f"chain1.{f}"
    rg, gr = r["regs"], g["regs"]
    assert np.array_equal(r["regs_off"], g["reg_off"])
    for i, f in enumerate(["rb", "re", "qb", "qe", "rid", "score", "truesc", "w", "seedcov", "seedlen0"]):
        assert np.array_equal(rg[f], gr[:, i]), f"reg.{f}"
    assert np.array_equal(rg["frac_rep"].view(np.int32), gr[:, 10].astype(np.int32))


@pytest.mark.parametrize("fn,genome", CASES, ids=[c[0] for c in CASES])
def test_oracle_chains_and_regions_match_reference(fn, genome, tmp_path_factory):
    bi = index_for(genome, tmp_path_factory)
    ob = oracle.OracleBwt(bi.primary, bi.L2[1:], bi.bwt, bi.sa, bi.sa_intv)
    anns = np.array([(a.offset, a.len, 0) for a in bi.anns], dtype=oracle.ANN_DTYPE)
    g = np.load(os.path.join(GOLDEN, fn))
    r = oracle.align_regs(ob, anns, bi.pac, bi.l_pac, oracle.Opt.from_list(g["opts"]), g["reads"],
                          g["read_off"], n_threads=4)
    check_against_golden(r, g)


def test_repeat_fixture_covers_hard_cases():
    g = np.load(os.path.join(GOLDEN, "reads_rep_L5.npz"))
    off, rows = g["chain0_off"], g["chain0_rows"]
    n = np.diff(off)
    assert n.max() > 45                       # several B-tree levels
    dup = sum(1 for r in range(len(n)) if len(set(rows[off[r]:off[r + 1], 5].tolist())) != n[r])
    assert dup > 10                           # equal chain keys


def check_dedup(r, g):
    assert np.array_equal(r[1], g["dedup_off"])
    d, gd = r[0], g["dedup"]
    for i, f in enumerate(["rb", "re", "qb", "qe", "rid", "score", "truesc", "w", "seedcov", "seedlen0", "n_comp"]):
        assert np.array_equal(d[f], gd[:, i]), f"dedup.{f}"
    assert np.array_equal(d["frac_rep"].view(np.int32), gd[:, 11].astype(np.int32))


@pytest.mark.parametrize("fn,genome", CASES, ids=[c[0] for c in CASES])
def test_oracle_dedup_matches_reference(fn, genome, tmp_path_factory):
    """mem_sort_dedup_patch on the reference's own pre-dedup regions gives the reference's
    post-dedup regions (sort orders, redundancy, merges with their global alignments)."""
    bi = index_for(genome, tmp_path_factory)
    g = np.load(os.path.join(GOLDEN, fn))
    pre = oracle.regs_from_golden(g["regs"])
    r = oracle.sort_dedup_batch(oracle.Opt.from_list(g["opts"]), bi.l_pac, bi.pac, g["reads"], g["read_off"], pre,
                                g["reg_off"])
    check_dedup(r, g)


def test_indel_fixture_covers_merges():
    g = np.load(os.path.join(GOLDEN, "reads_indel_W5.npz"))
    assert (g["dedup"][:, 10] > 1).sum() > 50                 # mem_patch_reg merges
    assert len(g["regs"]) - len(g["dedup"]) > 80              # regions dropped
