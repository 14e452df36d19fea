"""bsb_gen_cigar_batch (bwa_gen_cigar2 on the GPU) against the oracle and the reference.

Every record field (score, n_cigar, NM, the four methylation counts, status) and
every byte (CIGAR words, MD, XB) must be identical:
* to the reference's own records (tests/golden/cigar_*.npz), two scoring sets;
* to the oracle on the same job set including the statuses the reference cannot
  give (clipped context windows), and on a larger seeded set of reads from both
  strands of Watson and Crick contigs with indels, N bases and long bands.
"""
import os
import sys

import numpy as np
import pytest

import oracle
from bsbolt_gb300 import _lib, cigar, index, seed, synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import golden_data  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def loaded(gpu_ctx, tmp_path_factory):
    d = tmp_path_factory.mktemp("cigidx")
    fa = str(d / "ref.fa")
    synth.write_fasta(fa, golden_data.golden_genome())
    prefix = str(d / "ref")
    index.build_index(fa, prefix)
    seed.load_index(gpu_ctx, prefix)           # reads <prefix>.opac too
    return gpu_ctx, index.BwaIndex(prefix)


def opt_for(a, b, o_del, e_del, o_ins, e_ins):
    o = _lib.AlignOpt.bwa_defaults(a=a, b=b, o_del=o_del, e_del=e_del, o_ins=o_ins, e_ins=e_ins)
    return o


def assert_same(got, gblob, want, wblob, what):
    for f in ("status", "score", "n_cigar", "NM", "cg_meth", "cg_unmeth", "ch_meth", "ch_unmeth", "bytes", "off"):
        bad = np.nonzero(got[f] != want[f])[0]
        assert len(bad) == 0, f"{what}: {f} differs at jobs {bad[:8]}: {got[f][bad[:8]]} vs {want[f][bad[:8]]}"
    assert np.array_equal(gblob, wblob), f"{what}: record bytes differ"


@pytest.mark.parametrize("name", ["default", "asym"])
def test_gen_cigar_matches_reference_records(loaded, name):
    ctx, bi = loaded
    g = np.load(os.path.join(GOLDEN, f"cigar_{name}.npz"))
    a, b, o_del, e_del, o_ins, e_ins = (int(v) for v in g["scoring"])
    jobs, qbuf, obuf, tags = golden_data.golden_cigar_jobs(bi.pac, bi.opac, bi.l_pac, bi.crick_l)
    out, blob = cigar.gen_cigar_batch(ctx, jobs.view(cigar.JOB_DTYPE), qbuf, obuf, bi.crick_l,
                                      opt_for(a, b, o_del, e_del, o_ins, e_ins))
    keep = g["keep"]
    rec = g["recs"]
    o = out[keep]
    for i, f in enumerate(("score", "n_cigar", "NM", "cg_meth", "cg_unmeth", "ch_meth", "ch_unmeth", "status")):
        bad = np.nonzero(o[f] != rec[:, i])[0]
        assert len(bad) == 0, f"{f} differs for jobs {keep[bad[:5]]} ({tags[keep[bad[:5]]]})"
    for k, j in enumerate(keep):
        want = bytes(g["blob"][g["blob_off"][k]:g["blob_off"][k + 1]])
        got = bytes(blob[out["off"][j]:out["off"][j] + out["bytes"][j]])
        assert got == want, f"job {j} ({tags[j]}): {got!r} != {want!r}"
    # the jobs the reference cannot run get the oracle's status
    ref_o, _ = oracle.gen_cigar_batch(synth.fill_scmat(a, b), o_del, e_del, o_ins, e_ins, bi.l_pac, bi.pac,
                                      bi.opac, bi.crick_l, jobs, qbuf, obuf)
    assert np.array_equal(out["status"], ref_o["status"])


@pytest.mark.parametrize("scoring", [(1, 4, 6, 1, 6, 1), (2, 5, 5, 3, 7, 2), (1, 2, 3, 1, 2, 2)])
def test_gen_cigar_matches_oracle_random(loaded, scoring):
    ctx, bi = loaded
    jobs, qbuf, obuf, _ = golden_data.golden_cigar_jobs(bi.pac, bi.opac, bi.l_pac, bi.crick_l, n_random=4000,
                                                        seed=20261203 + 31 + scoring[2])
    a, b, o_del, e_del, o_ins, e_ins = scoring
    out, blob = cigar.gen_cigar_batch(ctx, jobs.view(cigar.JOB_DTYPE), qbuf, obuf, bi.crick_l,
                                      opt_for(a, b, o_del, e_del, o_ins, e_ins))
    ref, rblob = oracle.gen_cigar_batch(synth.fill_scmat(a, b), o_del, e_del, o_ins, e_ins, bi.l_pac, bi.pac,
                                        bi.opac, bi.crick_l, jobs, qbuf, obuf, n_threads=8)
    assert_same(out, blob, ref, rblob, f"scoring {scoring}")
    assert (out["status"] == cigar.OK).sum() > 3500
    assert (out["n_cigar"] > 3).sum() > 100


def test_gen_cigar_long_and_wide(loaded):
    """Reads up to the 1024-base limit, bands up to 400 (mem_reg2aln's opt->w << 2)."""
    ctx, bi = loaded
    rng = np.random.Generator(np.random.PCG64(5))
    jobs, qs, os_ = [], [], []
    qn = on = 0
    for k in range(300):
        L = int(rng.integers(200, 1025))
        rb = int(rng.integers(10, 2 * bi.l_pac - 1200))
        if rb < bi.l_pac < rb + L + 10:
            rb = bi.l_pac + 10
        ref = golden_data.doubled_seq(bi.pac, bi.l_pac, rb, rb + L)
        oref = golden_data.doubled_seq(bi.opac, bi.l_pac, rb, rb + L)
        q, oq = golden_data._edit(rng, [ref, oref], 0.02, int(rng.integers(0, 6)))
        q, oq = q[:1024], oq[:1024]
        re = rb + min(L + int(rng.integers(-5, 6)), 1024)
        w = int(rng.choice([5, 50, 100, 200, 400]))
        jobs.append((rb, re, qn, on, len(q), w))
        qs.append(q)
        os_.append(oq)
        qn += len(q)
        on += len(oq)
    jobs = np.array(jobs, cigar.JOB_DTYPE)
    qbuf, obuf = np.concatenate(qs), np.concatenate(os_)
    out, blob = cigar.gen_cigar_batch(ctx, jobs, qbuf, obuf, bi.crick_l)
    ref, rblob = oracle.gen_cigar_batch(synth.fill_scmat(1, 4), 6, 1, 6, 1, bi.l_pac, bi.pac, bi.opac, bi.crick_l,
                                        jobs, qbuf, obuf, n_threads=8)
    assert_same(out, blob, ref, rblob, "long reads")


def test_gen_cigar_errors(loaded):
    ctx, bi = loaded
    jobs, qbuf, obuf, _ = golden_data.golden_cigar_jobs(bi.pac, bi.opac, bi.l_pac, bi.crick_l, n_random=20)
    jobs = jobs.view(cigar.JOB_DTYPE)
    out, blob = cigar.gen_cigar_batch(ctx, jobs[:0], qbuf, obuf, bi.crick_l)           # empty batch
    assert len(out) == 0 and len(blob) == 0
    bad = jobs.copy()
    bad["qoff"][3] = len(qbuf)                                                          # query outside qbuf
    with pytest.raises(_lib.BsbError) as e:
        cigar.gen_cigar_batch(ctx, bad, qbuf, obuf, bi.crick_l)
    assert e.value.code == _lib.BSB_EINVAL
    bad = jobs.copy()
    bad["rb"][0], bad["re"][0] = 1000, 1000 + 1025                                      # over the length limit
    with pytest.raises(_lib.BsbError) as e:
        cigar.gen_cigar_batch(ctx, bad, qbuf, obuf, bi.crick_l)
    assert e.value.code == _lib.BSB_ETOOLONG
    with pytest.raises(_lib.BsbError) as e:
        cigar.upload_opac(ctx, bi.opac, bi.l_pac + 1)
    assert e.value.code == _lib.BSB_EINVAL
    # a valid batch after the errors still matches
    out, blob = cigar.gen_cigar_batch(ctx, jobs, qbuf, obuf, bi.crick_l)
    ref, rblob = oracle.gen_cigar_batch(synth.fill_scmat(1, 4), 6, 1, 6, 1, bi.l_pac, bi.pac, bi.opac, bi.crick_l,
                                        jobs, qbuf, obuf)
    assert_same(out, blob, ref, rblob, "after errors")
