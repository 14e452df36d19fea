"""Seeds -> chains -> chain filter -> mem_chain2aln on the GPU (bsb_align_regs_batch)
against the reference's pre-dedup regions (tests/golden/reads*_*.npz) and the
oracle, and with mem_sort_dedup_patch (bsb_mem_align1_batch) against the
reference's post-dedup regions and the oracle, through the C ABI.  Bit-exact,
including frac_rep's float bits."""
import os
import sys

import numpy as np
import pytest

import oracle
from bsbolt_gb300 import _lib, index, seed, synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import golden_data  # noqa: E402

pytestmark = pytest.mark.gpu

REG_FIELDS = ["rb", "re", "qb", "qe", "rid", "score", "truesc", "w", "seedcov", "seedlen0"]


def opt_from(o):
    o = [int(x) for x in o]
    return _lib.AlignOpt.bwa_defaults(a=o[0], b=o[1], o_del=o[2], e_del=o[3], o_ins=o[4], e_ins=o[5], w=o[6],
                                      zdrop=o[7], pen_clip5=o[8], pen_clip3=o[9], min_seed_len=o[10],
                                      max_occ=o[11], split_width=o[12], max_mem_intv=o[13], max_chain_gap=o[14])


@pytest.fixture(scope="module")
def indexes(tmp_path_factory):
    out = {}
    for tag, gen in (("plain", golden_data.golden_genome), ("rep", golden_data.golden_genome_rep)):
        d = tmp_path_factory.mktemp("aidx" + tag)
        synth.write_fasta(str(d / "ref.fa"), gen())
        index.build_index(str(d / "ref.fa"), str(d / "ref"))
        out[tag] = str(d / "ref")
    return out


GOLDEN_SETS = [("reads_L5.npz", "plain"), ("reads_L30.npz", "plain"), ("reads_rep_L5.npz", "rep"),
               ("reads_indel_W5.npz", "plain")]


@pytest.mark.parametrize("fn,tag", GOLDEN_SETS)
def test_regions_match_reference(gpu_ctx, indexes, fn, tag):
    seed.load_index(gpu_ctx, indexes[tag])
    g = np.load(os.path.join(GOLDEN, fn))
    regs, off = seed.align_regs(gpu_ctx, g["reads"], g["read_off"], opt_from(g["opts"]))
    assert np.array_equal(off, g["reg_off"]), "region counts per read differ"
    gr = g["regs"]
    for i, f in enumerate(REG_FIELDS):
        bad = np.nonzero(regs[f] != gr[:, i])[0]
        assert len(bad) == 0, f"{fn}: reg.{f} differs at {bad[:5]}"
    assert np.array_equal(regs["frac_rep"].view(np.int32), gr[:, 10].astype(np.int32))


@pytest.mark.parametrize("lmin,lmax", [(0, 127), (128, 159), (160, 255), (0, 300)],
                         ids=["up-to-127", "128-159", "160-255", "up-to-300"])
def test_regions_random_reads_vs_oracle(gpu_ctx, indexes, lmin, lmax):
    """Reads with errors and N runs, both strands, repeats; each length band runs a
    different chain-extension kernel variant (the batch's longest read picks it)."""
    prefix = indexes["rep"]
    seed.load_index(gpu_ctx, prefix)
    bi = index.BwaIndex(prefix)
    pac = bi.pac_codes()
    rng = np.random.Generator(np.random.PCG64(17 + lmin))
    reads = []
    for k in range(2500 if lmax == 300 else 1200):
        L = int(rng.integers(lmin, lmax + 1))
        st = int(rng.integers(0, len(pac) - L - 1))
        r = pac[st:st + L].copy()
        if k % 2:
            r = (3 - r[::-1]).astype(np.uint8)
        e = rng.random(L) < 0.03
        r[e] = rng.integers(0, 5, int(e.sum()))
        reads.append(r.astype(np.uint8))
    offs = np.zeros(len(reads) + 1, np.int64)
    offs[1:] = np.cumsum([len(r) for r in reads])
    seqs = np.concatenate(reads)
    opt = _lib.AlignOpt.bwa_defaults()
    regs, off = seed.align_regs(gpu_ctx, seqs, offs, opt)
    ob = oracle.OracleBwt(bi.primary, bi.L2[1:], bi.bwt, bi.sa, bi.sa_intv)
    anns = np.array([(a.offset, a.len, 0) for a in bi.anns], dtype=oracle.ANN_DTYPE)
    ref = oracle.align_regs(ob, anns, bi.pac, bi.l_pac,
                            oracle.Opt.from_list([1, 4, 6, 1, 6, 1, 100, 100, 5, 5, 19, 500, 10, 20, 10000]),
                            seqs, offs, n_threads=8)
    assert np.array_equal(off, ref["regs_off"])
    for f in REG_FIELDS + ["frac_rep"]:
        assert np.array_equal(regs[f], ref["regs"][f]), f"reg.{f}"


def test_align_rejects_reads_over_1023(gpu_ctx, indexes):
    seed.load_index(gpu_ctx, indexes["plain"])
    with pytest.raises(_lib.BsbError) as e:
        seed.align_regs(gpu_ctx, np.zeros(1024, np.uint8), np.array([0, 1024]))
    assert e.value.code == _lib.BSB_ETOOLONG


@pytest.mark.parametrize("mcw,lmin,lmax,n", [(0, 513, 1023, 600), (5, 100, 300, 1500), (0, 700, 760, 400)],
                         ids=["long-reads", "W5", "filter-threshold"])
def test_long_reads_and_seed_sw_filter_vs_oracle(gpu_ctx, indexes, mcw, lmin, lmax, n):
    """Reads up to 1023 bases (the 32-column chain-extension width) and the seed-level
    Smith-Waterman filter of mem_flt_chained_seeds (bwamem.c:602-619): it runs where
    5.5*ln(L) <= 0.05*L (from ~724 bases) with -W 0, and from 22*W bases with -W W.  Regions
    before and after mem_sort_dedup_patch against the oracle."""
    prefix = indexes["rep"]
    seed.load_index(gpu_ctx, prefix)
    bi = index.BwaIndex(prefix)
    pac = bi.pac_codes()
    rng = np.random.Generator(np.random.PCG64(29 + mcw + lmin))
    reads = []
    for k in range(n):
        L = int(rng.integers(lmin, lmax + 1))
        st = int(rng.integers(0, len(pac) - L - 1))
        r = pac[st:st + L].copy()
        if k % 2:
            r = (3 - r[::-1]).astype(np.uint8)
        e = rng.random(L) < (0.03 if k % 3 else 0.12)          # some reads with weak seeds
        r[e] = rng.integers(0, 5, int(e.sum()))
        reads.append(r.astype(np.uint8))
    offs = np.zeros(len(reads) + 1, np.int64)
    offs[1:] = np.cumsum([len(r) for r in reads])
    seqs = np.concatenate(reads)
    opt = _lib.AlignOpt.bwa_defaults()
    opt.min_chain_weight = mcw
    ob = oracle.OracleBwt(bi.primary, bi.L2[1:], bi.bwt, bi.sa, bi.sa_intv)
    anns = np.array([(a.offset, a.len, 0) for a in bi.anns], dtype=oracle.ANN_DTYPE)
    oo = oracle.Opt.from_list([1, 4, 6, 1, 6, 1, 100, 100, 5, 5, 19, 500, 10, 20, 10000])
    oo.min_chain_weight = mcw
    ref = oracle.align_regs(ob, anns, bi.pac, bi.l_pac, oo, seqs, offs, n_threads=8)
    regs, off = seed.align_regs(gpu_ctx, seqs, offs, opt)
    assert np.array_equal(off, ref["regs_off"])
    for f in REG_FIELDS + ["frac_rep"]:
        assert np.array_equal(regs[f], ref["regs"][f]), f"reg.{f}"
    dregs, doff = seed.align_regs(gpu_ctx, seqs, offs, opt, dedup=True)
    dref, dref_off = oracle.sort_dedup_batch(oo, bi.l_pac, bi.pac, seqs, offs, ref["regs"], ref["regs_off"])
    assert np.array_equal(doff, dref_off)
    for f in dref.dtype.names:
        assert np.array_equal(dregs[f], dref[f]), f"dedup.{f}"


@pytest.mark.parametrize("fn,tag", GOLDEN_SETS)
def test_dedup_regions_match_reference(gpu_ctx, indexes, fn, tag):
    """bsb_mem_align1_batch: the regions mem_align1_core returns (after mem_sort_dedup_patch),
    including merged regions (n_comp, the merge's global-alignment score) in the indel set."""
    seed.load_index(gpu_ctx, indexes[tag])
    g = np.load(os.path.join(GOLDEN, fn))
    regs, off = seed.align_regs(gpu_ctx, g["reads"], g["read_off"], opt_from(g["opts"]), dedup=True)
    assert np.array_equal(off, g["dedup_off"]), "region counts per read differ"
    gd = g["dedup"]
    for i, f in enumerate(REG_FIELDS + ["n_comp"]):
        bad = np.nonzero(regs[f] != gd[:, i])[0]
        assert len(bad) == 0, f"{fn}: dedup.{f} differs at {bad[:5]}"
    assert np.array_equal(regs["frac_rep"].view(np.int32), gd[:, 11].astype(np.int32))


def test_dedup_random_indel_reads_vs_oracle(gpu_ctx, indexes):
    """Reads of 150-300 bases with indels and duplicated stretches at band 5 and 10 (merges),
    both strands, against the oracle's mem_sort_dedup_patch on the oracle's own regions."""
    prefix = indexes["plain"]
    seed.load_index(gpu_ctx, prefix)
    bi = index.BwaIndex(prefix)
    reads = golden_data.golden_reads_indel(n=1500, seed=20261203 + 71)
    offs = np.zeros(len(reads) + 1, np.int64)
    offs[1:] = np.cumsum([len(r) for r in reads])
    seqs = np.concatenate(reads)
    ob = oracle.OracleBwt(bi.primary, bi.L2[1:], bi.bwt, bi.sa, bi.sa_intv)
    anns = np.array([(a.offset, a.len, 0) for a in bi.anns], dtype=oracle.ANN_DTYPE)
    merged = 0
    for w in (5, 10):
        o = [1, 4, 6, 1, 6, 1, w, 100, 5, 5, 19, 500, 10, 20, 10000]
        regs, off = seed.align_regs(gpu_ctx, seqs, offs, opt_from(o), dedup=True)
        oo = oracle.Opt.from_list(o)
        pre = oracle.align_regs(ob, anns, bi.pac, bi.l_pac, oo, seqs, offs, n_threads=8)
        ref, ref_off = oracle.sort_dedup_batch(oo, bi.l_pac, bi.pac, seqs, offs, pre["regs"], pre["regs_off"])
        assert np.array_equal(off, ref_off)
        for f in REG_FIELDS + ["n_comp", "frac_rep"]:
            assert np.array_equal(regs[f], ref[f]), f"w={w}: dedup.{f}"
        merged += int((regs["n_comp"] > 1).sum())
    assert merged > 100


def test_learned_read_order_changes_no_region(gpu_ctx, indexes):
    """The per-read log (features, DP cells of the read's ksw_extend2 calls) and the learned
    read order: the logged cells add up to the oracle's cell count of the same reads, a model
    trained on the log orders the reads, and the regions stay the same."""
    torch = pytest.importorskip("torch")
    from bsbolt_gb300 import cost_model as cm
    prefix = indexes["rep"]
    seed.load_index(gpu_ctx, prefix)
    g = np.load(os.path.join(GOLDEN, "reads_rep_L5.npz"))
    reads, offs = g["reads"], g["read_off"]
    n = len(offs) - 1
    opt = opt_from(g["opts"])
    seed.read_cost_log(gpu_ctx, True)
    try:
        plain, plain_off = seed.align_regs(gpu_ctx, reads, offs, opt, dedup=True)
        feat, cells = seed.last_read_costs(gpu_ctx, n)
    finally:
        seed.read_cost_log(gpu_ctx, False)
    bi = index.BwaIndex(prefix)
    ob = oracle.OracleBwt(bi.primary, bi.L2[1:], bi.bwt, bi.sa, bi.sa_intv)
    anns = np.array([(a.offset, a.len, 0) for a in bi.anns], dtype=oracle.ANN_DTYPE)
    ref = oracle.align_regs(ob, anns, bi.pac, bi.l_pac, oracle.Opt.from_list([int(x) for x in g["opts"]]), reads,
                            offs, n_threads=8)
    assert int(cells.sum()) == int(ref["cells"]) and np.isfinite(feat).all() and (cells >= 0).all()
    model = cm.CostModel(gpu_ctx, seed=3)
    model.train(torch.from_numpy(feat).cuda(), torch.from_numpy(np.log1p(cells).astype(np.float32)).cuda(),
                epochs=3, batch=64)
    seed.set_read_cost_model(gpu_ctx, model)
    try:
        learned, learned_off = seed.align_regs(gpu_ctx, reads, offs, opt, dedup=True)
    finally:
        seed.set_read_cost_model(gpu_ctx, None)
    assert np.array_equal(plain_off, learned_off) and np.array_equal(plain, learned)
    # the exact-cost order (the logged cells as keys, once) and the reverse of it
    for keys in (cells, -cells):
        seed.set_read_order_keys(gpu_ctx, keys)
        exact, exact_off = seed.align_regs(gpu_ctx, reads, offs, opt, dedup=True)
        assert np.array_equal(plain_off, exact_off) and np.array_equal(plain, exact)


def test_stage_times_of_the_last_batch(gpu_ctx, indexes):
    """bsb_last_stage_ms: six non-negative stage times of the last alignment batch whose sum
    is within the host's wall time of that call."""
    import time
    seed.load_index(gpu_ctx, indexes["plain"])
    g = np.load(os.path.join(GOLDEN, "reads_L5.npz"))
    t0 = time.perf_counter()
    seed.align_regs(gpu_ctx, g["reads"], g["read_off"], opt_from(g["opts"]), dedup=True)
    wall_ms = (time.perf_counter() - t0) * 1e3
    st = seed.last_stage_ms(gpu_ctx)
    assert list(st) == list(seed.ALIGN_STAGES)
    assert all(v >= 0 for v in st.values()) and st["seeding"] > 0 and st["chain2aln"] > 0
    assert sum(st.values()) <= wall_ms + 1.0
