"""SMEM seeding and SA lookups on the GPU against the reference's seed lists
(tests/golden/reads_*.npz) and the oracle, through the C ABI.  Bit-exact."""
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


@pytest.fixture(scope="module")
def idx(tmp_path_factory):
    d = tmp_path_factory.mktemp("gidx")
    fa = str(d / "ref.fa")
    synth.write_fasta(fa, golden_data.golden_genome())
    prefix = str(d / "ref")
    index.build_index(fa, prefix)
    return prefix


@pytest.fixture(scope="module")
def ctx_idx(gpu_ctx, idx):
    seed.load_index(gpu_ctx, idx)
    return gpu_ctx


@pytest.mark.parametrize("name", ["L5", "L30"])
def test_seeds_match_reference(ctx_idx, name):
    d = np.load(os.path.join(GOLDEN, f"reads_{name}.npz"))
    o = d["opts"]
    got, off = seed.seed_batch(ctx_idx, d["reads"], d["read_off"], min_seed_len=int(o[10]),
                               split_width=int(o[12]), max_mem_intv=int(o[13]))
    ref, roff = d["smem"], d["smem_off"]
    lens = d["read_off"][1:] - d["read_off"][:-1]
    for r in range(len(lens)):
        exp = ref[roff[r]:roff[r + 1]] if lens[r] >= int(o[10]) else ref[0:0]
        assert np.array_equal(got[off[r]:off[r + 1]], exp), f"read {r}: seeds differ"


def test_seeds_random_reads_vs_oracle(ctx_idx, idx):
    """Reads with errors, N runs, repeats and every length 0..300 against the oracle."""
    bi = index.BwaIndex(idx)
    pac = bi.pac_codes()
    rng = np.random.Generator(np.random.PCG64(11))
    reads = []
    for k in range(3000):
        L = int(rng.integers(0, 301)) if k % 3 else 150
        st = int(rng.integers(0, len(pac) - L - 1))
        r = pac[st:st + L].copy()
        if k % 2:
            r = (3 - r[::-1]).astype(np.uint8)
        e = rng.random(L) < 0.02
        r[e] = rng.integers(0, 5, int(e.sum()))
        reads.append(r.astype(np.uint8))
    offs = np.zeros(len(reads) + 1, np.int64)
    offs[1:] = np.cumsum([len(r) for r in reads])
    seqs = np.concatenate(reads)
    got, off = seed.seed_batch(ctx_idx, seqs, offs)
    ob = oracle.OracleBwt(bi.primary, bi.L2[1:], bi.bwt, bi.sa, bi.sa_intv)
    exp, eoff = ob.collect_intv(seqs, offs, n_threads=8)
    assert np.array_equal(off, eoff)
    assert np.array_equal(got, exp)


@pytest.mark.parametrize("resident", [True, False], ids=["full-sa", "lf-walk"])
def test_sa_lookup_vs_suffix_array(ctx_idx, idx, resident):
    """Every row, with the full suffix array resident and with the reference's LF walk."""
    bi = index.BwaIndex(idx)
    pac = bi.pac_codes()
    text = np.concatenate([pac, 3 - pac[::-1]]).astype(np.uint8)
    full = index.suffix_array(text).astype(np.int64)
    rows = np.arange(0, len(full)).astype(np.uint64)
    _lib.check(ctx_idx.handle, ctx_idx.L.bsb_index_full_sa(ctx_idx.handle, int(resident)))
    try:
        got = seed.sa_batch(ctx_idx, rows).astype(np.int64)
    finally:
        _lib.check(ctx_idx.handle, ctx_idx.L.bsb_index_full_sa(ctx_idx.handle, 1))
    exp = np.where(full == len(text), -1, full)
    assert np.array_equal(got, exp)


def test_seed_errors(gpu_ctx, ctx_idx):
    with pytest.raises(_lib.BsbError) as e:
        seed.seed_batch(ctx_idx, np.zeros(2000, np.uint8), np.array([0, 2000]))
    assert e.value.code == _lib.BSB_ETOOLONG
    with pytest.raises(_lib.BsbError) as e:
        seed.sa_batch(ctx_idx, np.array([1 << 60], np.uint64))
    assert e.value.code == _lib.BSB_EINVAL


@pytest.mark.parametrize("sym64", ["1", "0"], ids=["64-symbol-sectors", "32-symbol-sectors"])
def test_occurrence_layouts_give_the_same_seeds_and_sa(gpu_ctx, idx, monkeypatch, sym64):
    """The two device layouts of the occurrence array (32-symbol sectors, 64-symbol sectors with
    2^32-row superblocks), forced at upload: seed lists against the reference's own (golden
    L5 set) and the oracle, and every SA row through the LF walk and the full SA built from it."""
    from bsbolt_gb300 import extend
    monkeypatch.setenv("BSB_OCC_SYM64", sym64)
    ctx = extend.Context(0)
    try:
        seed.load_index(ctx, idx)
        d = np.load(os.path.join(GOLDEN, "reads_L5.npz"))
        o = d["opts"]
        got, off = seed.seed_batch(ctx, d["reads"], d["read_off"], min_seed_len=int(o[10]),
                                   split_width=int(o[12]), max_mem_intv=int(o[13]))
        ref, roff = d["smem"], d["smem_off"]
        lens = d["read_off"][1:] - d["read_off"][:-1]
        for r in range(len(lens)):
            exp = ref[roff[r]:roff[r + 1]] if lens[r] >= int(o[10]) else ref[0:0]
            assert np.array_equal(got[off[r]:off[r + 1]], exp), f"read {r}: seeds differ"
        bi = index.BwaIndex(idx)
        pac = bi.pac_codes()
        text = np.concatenate([pac, 3 - pac[::-1]]).astype(np.uint8)
        full = index.suffix_array(text).astype(np.int64)
        want = np.where(full == len(text), -1, full)
        rows = np.arange(0, len(full)).astype(np.uint64)
        for resident in (1, 0):
            _lib.check(ctx.handle, ctx.L.bsb_index_full_sa(ctx.handle, resident))
            assert np.array_equal(seed.sa_batch(ctx, rows).astype(np.int64), want)
    finally:
        ctx.close()


def test_seed_slots_grow_for_reads_with_many_seeds(ctx_idx, idx):
    """min_seed_len 8 and split_width 3 give some reads more SMEMs and re-seeds than their
    2*len + 32 seed slots: the batch runs again with more slots per read (seeding and the
    alignment batch alike), and the seeds and regions equal the oracle's."""
    bi = index.BwaIndex(idx)
    pac = bi.pac_codes()
    rng = np.random.Generator(np.random.PCG64(71))
    reads = []
    for k in range(1500):
        L = int(rng.integers(1, 160))
        st = int(rng.integers(0, len(pac) - L - 1))
        r = pac[st:st + L].copy()
        if k % 2:
            r = (3 - r[::-1]).astype(np.uint8)
        e = rng.random(L) < 0.02
        r[e] = rng.integers(0, 4, int(e.sum()))
        if k % 5 == 0 and L > 20:
            p = int(rng.integers(0, L - 5))
            r[p:p + int(rng.integers(1, 5))] = 4
        reads.append(r.astype(np.uint8))
    offs = np.zeros(len(reads) + 1, np.int64)
    offs[1:] = np.cumsum([len(r) for r in reads])
    seqs = np.concatenate(reads)
    ob = oracle.OracleBwt(bi.primary, bi.L2[1:], bi.bwt, bi.sa, bi.sa_intv)
    got, off = seed.seed_batch(ctx_idx, seqs, offs, min_seed_len=8, split_width=3, max_mem_intv=50)
    ref, roff = ob.collect_intv(seqs, offs, min_seed_len=8, split_width=3, max_mem_intv=50, n_threads=8)
    lens = offs[1:] - offs[:-1]
    assert ((roff[1:] - roff[:-1]) > 1.5 * lens + 24).any(), "no read needs more than its first slots"
    assert np.array_equal(off, roff) and np.array_equal(got, ref)
    o = [1, 4, 6, 1, 6, 1, 100, 100, 5, 5, 8, 500, 3, 50, 10000]
    opt = _lib.AlignOpt.bwa_defaults(min_seed_len=8, split_width=3, max_mem_intv=50)
    regs, roff2 = seed.align_regs(ctx_idx, seqs, offs, opt)
    anns = np.array([(a.offset, a.len, 0) for a in bi.anns], dtype=oracle.ANN_DTYPE)
    want = oracle.align_regs(ob, anns, bi.pac, bi.l_pac, oracle.Opt.from_list(o), seqs, offs, n_threads=8)
    assert np.array_equal(roff2, want["regs_off"])
    for f in want["regs"].dtype.names:
        assert np.array_equal(regs[f], want["regs"][f]), f"reg.{f}"
