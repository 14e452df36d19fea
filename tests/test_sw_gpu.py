"""bsb_align2_batch (ksw_align2 on the GPU) against the reference and the oracle.

Every kswr_t field must be identical: to the reference's own results
(tests/golden/sw_*.npz, three scoring sets, byte and word lanes, every flag
combination), and to the oracle on a larger seeded set of mate-rescue-shaped jobs."""
import os
import sys

import numpy as np
import pytest

import oracle
from bsbolt_gb300 import _lib, matesw, synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import golden_data  # noqa: E402

pytestmark = pytest.mark.gpu
FIELDS = ("score", "te", "qe", "score2", "te2", "tb", "qb")


def assert_same(got, want, tags, what):
    for f in FIELDS:
        w = want[f] if want.dtype.names else want[:, FIELDS.index(f)]
        bad = np.nonzero(got[f] != w)[0]
        assert len(bad) == 0, f"{what}: {f} differs at jobs {bad[:6]} ({tags[bad[:6]] if tags is not None else ''}): " \
                              f"{got[f][bad[:6]]} vs {w[bad[:6]]}"


@pytest.mark.parametrize("name", ["default", "asym", "wide"])
def test_align2_matches_reference(gpu_ctx, name):
    g = np.load(os.path.join(GOLDEN, f"sw_{name}.npz"))
    a, b, o_del, e_del, o_ins, e_ins = (int(v) for v in g["scoring"])
    jobs, seq, tags = golden_data.golden_sw_jobs(a)
    out = matesw.align2_batch(gpu_ctx, jobs.view(matesw.JOB_DTYPE), seq, synth.fill_scmat(a, b), o_del, e_del,
                              o_ins, e_ins)
    assert_same(out, g["recs"], tags, name)


@pytest.mark.parametrize("seed", [1, 2])
def test_align2_matches_oracle_random(gpu_ctx, seed):
    jobs, seq, tags = golden_data.golden_sw_jobs(1, n=6000, seed=20261203 + 40 + seed)
    mat = synth.fill_scmat(1, 4)
    out = matesw.align2_batch(gpu_ctx, jobs.view(matesw.JOB_DTYPE), seq, mat, 6, 1, 6, 1)
    ref = oracle.align2_batch(jobs, seq, mat, 6, 1, 6, 1, n_threads=8)
    assert_same(out, ref, tags, f"seed {seed}")
    assert (out["score2"] > 0).sum() > 300 and (out["tb"] >= 0).sum() > 2000


def test_align2_errors(gpu_ctx):
    jobs, seq, _ = golden_data.golden_sw_jobs(1, n=20)
    jobs = jobs.view(matesw.JOB_DTYPE)
    mat = synth.fill_scmat(1, 4)
    assert len(matesw.align2_batch(gpu_ctx, jobs[:0], seq, mat, 6, 1, 6, 1)) == 0
    bad = jobs.copy()
    bad["toff"][2] = len(seq)
    with pytest.raises(_lib.BsbError) as e:
        matesw.align2_batch(gpu_ctx, bad, seq, mat, 6, 1, 6, 1)
    assert e.value.code == _lib.BSB_EINVAL
    long_q = np.zeros(1100, np.uint8)
    lj = np.array([(0, 0, 1100, 100, matesw.KSW_XSTART, 0)], matesw.JOB_DTYPE)
    with pytest.raises(_lib.BsbError) as e:
        matesw.align2_batch(gpu_ctx, lj, long_q, mat, 6, 1, 6, 1)
    assert e.value.code == _lib.BSB_ETOOLONG
    with pytest.raises(_lib.BsbError) as e:
        matesw.align2_batch(gpu_ctx, jobs, seq, -np.abs(mat), 6, 1, 6, 1)
    assert e.value.code == _lib.BSB_EINVAL
    out = matesw.align2_batch(gpu_ctx, jobs, seq, mat, 6, 1, 6, 1)
    ref = oracle.align2_batch(jobs, seq, mat, 6, 1, 6, 1)
    assert_same(out, ref, None, "after errors")


@pytest.mark.parametrize("scoring", [(2, 3, 5, 2, 7, 1), (1, 4, 0, 1, 0, 1), (1, 4, 6, 0, 6, 0),
                                     (1, 4, 6, 1, 250, 10), (2, 3, 255, 255, 255, 255), (5, 3, 100, 50, 120, 60),
                                     (1, 4, 20000, 9000, 30000, 3000)])
def test_align2_scorings_match_oracle(gpu_ctx, scoring):
    """Other scorings: asymmetric, zero open or extension penalties, byte-lane penalties that
    wrap (o + e >= 256: the one-lane kernels keep the reference's lazy-F loop), penalties that
    keep word lanes off the 16-bit path."""
    a, b, o_del, e_del, o_ins, e_ins = scoring
    jobs, seq, tags = golden_data.golden_sw_jobs(a, n=2500, seed=20261203 + 60 + a + o_ins)
    mat = synth.fill_scmat(a, b)
    out = matesw.align2_batch(gpu_ctx, jobs.view(matesw.JOB_DTYPE), seq, mat, o_del, e_del, o_ins, e_ins)
    ref = oracle.align2_batch(jobs, seq, mat, o_del, e_del, o_ins, e_ins, n_threads=8)
    assert_same(out, ref, tags, f"scoring {scoring}")


@pytest.mark.parametrize("a,lo,hi", [(1, 250, 330), (2, 125, 200)])
def test_align2_long_word_lane_mates(gpu_ctx, a, lo, hi):
    """Mates too long for byte lanes (qlen * a >= 250): word lanes of 17-42 segments, the
    packed kernels up to 40 segments (320 bases) and the one-lane kernel beyond."""
    rng = np.random.Generator(np.random.PCG64(20261203 + 90 + a))
    jobs, parts, off = [], [], 0
    for k in range(1500):
        L = int(rng.integers(lo, hi + 1))
        q = rng.integers(0, 4, L).astype(np.uint8)
        wl = int(rng.integers(L + 20, L + 500))
        t = rng.integers(0, 4, wl).astype(np.uint8)
        if k % 4:
            m = q.copy()
            sub = rng.random(L) < 0.05
            m[sub] = rng.integers(0, 4, int(sub.sum()))
            at = int(rng.integers(0, wl - L + 1))
            t[at:at + L] = m
        xtra = matesw.matesw_xtra(L, a)
        jobs.append((off, off + L, L, wl, xtra, 0))
        parts += [q, t]
        off += L + wl
    jobs = np.array(jobs, matesw.JOB_DTYPE)
    seq = np.concatenate(parts)
    assert not (jobs["xtra"] & matesw.KSW_XBYTE).any()
    mat = synth.fill_scmat(a, 4)
    out = matesw.align2_batch(gpu_ctx, jobs, seq, mat, 6, 1, 6, 1)
    ref = oracle.align2_batch(jobs.view(golden_data.SW_JOB_DTYPE), seq, mat, 6, 1, 6, 1, n_threads=8)
    assert_same(out, ref, None, f"a={a} qlen {lo}-{hi}")
    assert (out["tb"] >= 0).sum() > 800
