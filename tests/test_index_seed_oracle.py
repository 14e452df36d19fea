"""Index builder, oracle seeding and oracle SA lookup against the reference (CPU only).

* the host SA-IS index builder reproduces the reference `bwa index` files
  byte for byte (tests/golden/index_sha256.json);
* the oracle's mem_collect_intv reproduces the reference's seed lists
  (tests/golden/reads_*.npz, captured from mem_chain's smem buffer);
* the oracle's bwt_sa agrees with the full suffix array;
* the oracle's ksw_extend2 reproduces every extension the reference ran
  inside mem_chain2aln for those reads.
"""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

import oracle
from bsbolt_gb300 import index, synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import golden_data  # noqa: E402


@pytest.fixture(scope="module")
def idx(tmp_path_factory):
    d = tmp_path_factory.mktemp("idx")
    fa = str(d / "ref.fa")
    synth.write_fasta(fa, golden_data.golden_genome())
    prefix = str(d / "ref")
    index.build_index(fa, prefix)
    return prefix


def sha(fn):
    return hashlib.sha256(open(fn, "rb").read()).hexdigest()


def test_index_files_match_reference(idx):
    want = json.load(open(os.path.join(GOLDEN, "index_sha256.json")))["files"]
    for ext, h in want.items():
        assert sha(idx + "." + ext) == h, f".{ext} differs from the reference bwa index"


def test_repeat_index_files_match_reference(tmp_path):
    fa = str(tmp_path / "rep.fa")
    synth.write_fasta(fa, golden_data.golden_genome_rep())
    index.build_index(fa, str(tmp_path / "rep"))
    want = json.load(open(os.path.join(GOLDEN, "index_rep_sha256.json")))["files"]
    for ext, h in want.items():
        assert sha(str(tmp_path / "rep") + "." + ext) == h, f".{ext} differs from the reference bwa index"


def test_suffix_array_small_exhaustive():
    rng = np.random.Generator(np.random.PCG64(1))
    for n in list(range(1, 40)) + [200, 1000]:
        for alpha in (1, 2, 4):
            t = rng.integers(0, alpha, n).astype(np.uint8)
            sa = index.suffix_array(t)
            ref = sorted(range(n + 1), key=lambda i: list(t[i:]) + [-1])
            assert sa.tolist() == ref


def oracle_bwt(bi):
    return oracle.OracleBwt(bi.primary, bi.L2[1:], bi.bwt, bi.sa, bi.sa_intv)


@pytest.mark.parametrize("name", ["L5", "L30"])
def test_oracle_seeds_match_reference(idx, name):
    d = np.load(os.path.join(GOLDEN, f"reads_{name}.npz"))
    bi = index.BwaIndex(idx)
    ob = oracle_bwt(bi)
    o = d["opts"]
    seeds, off = ob.collect_intv(d["reads"], d["read_off"], min_seed_len=int(o[10]),
                                 split_width=int(o[12]), max_mem_intv=int(o[13]), n_threads=4)
    ref, roff = d["smem"], d["smem_off"]
    lens = d["read_off"][1:] - d["read_off"][:-1]
    for r in range(len(lens)):
        got = seeds[off[r]:off[r + 1]]
        exp = ref[roff[r]:roff[r + 1]] if lens[r] >= int(o[10]) else ref[0:0]
        assert np.array_equal(got, exp), f"read {r}: seeds differ"


def test_oracle_sa_matches_suffix_array(idx):
    bi = index.BwaIndex(idx)
    ob = oracle_bwt(bi)
    pac = bi.pac_codes()
    text = np.concatenate([pac, 3 - pac[::-1]]).astype(np.uint8)
    full = index.suffix_array(text).astype(np.int64)
    rng = np.random.Generator(np.random.PCG64(2))
    rows = np.concatenate([np.arange(0, 70), rng.integers(0, len(full), 5000)]).astype(np.uint64)
    got = ob.sa_lookup(rows).astype(np.int64)
    exp = full[rows.astype(np.int64)]
    exp = np.where(exp == len(text), -1, exp)       # row 0 is the $ suffix: sa[0] = -1 (bwt.c:83)
    assert np.array_equal(got, exp)


@pytest.mark.parametrize("name", ["L5", "L30"])
def test_oracle_ksw_matches_reference_job_stream(name):
    d = np.load(os.path.join(GOLDEN, f"reads_{name}.npz"))
    h, ref, seq, so = d["ksw_hdr"], d["ksw_out"], d["ksw_seq"], d["ksw_seq_off"]
    assert len(h) > 100
    jobs = np.zeros(len(h), synth.JOB_DTYPE)
    jobs["qoff"] = so[:-1]
    jobs["toff"] = so[:-1] + h[:, 1]
    jobs["qlen"], jobs["tlen"], jobs["h0"], jobs["w"], jobs["end_bonus"] = h[:, 1], h[:, 2], h[:, 3], h[:, 4], h[:, 5]
    o = d["opts"]
    out, _ = oracle.ksw_batch(jobs, seq, synth.fill_scmat(int(o[0]), int(o[1])), int(o[2]), int(o[3]),
                              int(o[4]), int(o[5]), int(o[7]))
    assert np.array_equal(out, ref)


def test_bwt_sa_writer_from_a_64bit_suffix_array(tmp_path):
    """The writer the GPU-sorted suffix array goes through (bsbh_write_bwt_sa64), fed the host
    SA-IS order as int64, gives the reference `bwa index` files byte for byte."""
    import ctypes
    fa = str(tmp_path / "ref.fa")
    synth.write_fasta(fa, golden_data.golden_genome())
    prefix = str(tmp_path / "ref")
    L = index.host_lib()
    l_pac = ctypes.c_int64()
    assert L.bsbh_index_fasta_nobwt(fa.encode(), prefix.encode(), ctypes.byref(l_pac)) == 0
    n = l_pac.value
    pac = np.fromfile(prefix + ".pac", dtype=np.uint8)[: (n + 3) // 4].copy()
    b = ((pac[np.arange(n) >> 2] >> ((~np.arange(n) & 3) << 1)) & 3).astype(np.uint8)
    sa = index.suffix_array(np.concatenate([b, 3 - b[::-1]]).astype(np.uint8)).astype(np.int64)
    assert L.bsbh_write_bwt_sa64(prefix.encode(), pac.ctypes.data_as(ctypes.c_void_p), n,
                                 sa.ctypes.data_as(ctypes.c_void_p), 32) == 0
    want = json.load(open(os.path.join(GOLDEN, "index_sha256.json")))["files"]
    for ext, h in want.items():
        assert sha(prefix + "." + ext) == h, f".{ext} differs from the reference bwa index"


def test_bwt_writer_from_a_packed_bwt(tmp_path):
    """The writer bsb_build_bwt's output goes through (bsbh_write_bwt_packed): the BWT packed 16
    symbols to a word without the row of suffix 0, that row, and every 32nd suffix-array row,
    here derived from the host SA-IS order, give the reference `bwa index` files byte for byte."""
    import ctypes
    fa = str(tmp_path / "ref.fa")
    synth.write_fasta(fa, golden_data.golden_genome())
    prefix = str(tmp_path / "ref")
    L = index.host_lib()
    l_pac = ctypes.c_int64()
    assert L.bsbh_index_fasta_nobwt(fa.encode(), prefix.encode(), ctypes.byref(l_pac)) == 0
    n = l_pac.value
    pac = np.fromfile(prefix + ".pac", dtype=np.uint8)[: (n + 3) // 4].copy()
    b = ((pac[np.arange(n) >> 2] >> ((~np.arange(n) & 3) << 1)) & 3).astype(np.uint8)
    text = np.concatenate([b, 3 - b[::-1]]).astype(np.uint8)
    sa = index.suffix_array(text).astype(np.int64)
    primary = int(np.nonzero(sa == 0)[0][0])
    sym = text[sa[sa != 0] - 1].astype(np.uint32)
    sym = np.concatenate([sym, np.zeros((-len(sym)) % 16, np.uint32)]).reshape(-1, 16)
    words = np.zeros(len(sym), np.uint32)
    for j in range(16):
        words |= sym[:, j] << np.uint32((15 - j) * 2)
    samples = sa[::32].astype(np.uint64)
    assert len(samples) == (2 * n + 32) // 32
    assert L.bsbh_write_bwt_packed(prefix.encode(), 2 * n, words.ctypes.data_as(ctypes.c_void_p), primary,
                                   samples.ctypes.data_as(ctypes.c_void_p), 32) == 0
    want = json.load(open(os.path.join(GOLDEN, "index_sha256.json")))["files"]
    for ext, h in want.items():
        assert sha(prefix + "." + ext) == h, f".{ext} differs from the reference bwa index"
