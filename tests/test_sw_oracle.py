"""Mate-rescue Smith-Waterman oracle against the reference's own ksw_align2 (CPU only).

tests/golden/sw_*.npz hold the reference's kswr_t results (score, te, qe, score2,
te2, tb, qb) for seeded mem_matesw-shaped jobs and the corner cases of the interface,
in three scoring sets (one with gap penalties that the byte lanes truncate, as the
reference does); the oracle's restatement of the striped algorithm must reproduce
every field."""
import os
import sys

import numpy as np
import pytest

import oracle
from bsbolt_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import golden_data  # noqa: E402

FIELDS = ("score", "te", "qe", "score2", "te2", "tb", "qb")


@pytest.mark.parametrize("name", ["default", "asym", "wide"])
def test_oracle_align2_matches_reference(name):
    g = np.load(os.path.join(GOLDEN, f"sw_{name}.npz"))
    a, b, o_del, e_del, o_ins, e_ins = (int(v) for v in g["scoring"])
    jobs, seq, tags = golden_data.golden_sw_jobs(a)
    out = oracle.align2_batch(jobs, seq, synth.fill_scmat(a, b), o_del, e_del, o_ins, e_ins, n_threads=8)
    rec = g["recs"]
    for i, f in enumerate(FIELDS):
        bad = np.nonzero(out[f] != rec[:, i])[0]
        assert len(bad) == 0, f"{f} differs at jobs {bad[:6]} ({tags[bad[:6]]}): {out[f][bad[:6]]} vs {rec[bad[:6], i]}"
    # the set exercises suboptimal hits, start positions and both lane widths
    assert (rec[:, 3] > 0).sum() > 100 and (rec[:, 5] >= 0).sum() > 300
    assert (jobs["xtra"] & oracle.KSW_XBYTE).sum() > 100 and (~jobs["xtra"] & oracle.KSW_XBYTE).sum() > 100


@pytest.mark.parametrize("scoring", [(1, 4, 6, 1, 6, 1), (2, 5, 5, 2, 7, 1), (1, 4, 0, 1, 0, 1), (1, 4, 6, 0, 6, 0),
                                     (3, 2, 1, 3, 2, 4), (5, 3, 100, 50, 120, 60)])
def test_closed_form_lazy_f_matches_the_loop(scoring, tmp_path):
    """The lazy-F loop in closed form (a max-plus scan over the lanes, then one max per
    segment), as the GPU kernels run it, gives every kswr_t field the reference's loop gives:
    the oracle built with -DORC_SW_LAZY_F_CLOSED_FORM against the default oracle."""
    import ctypes
    import subprocess
    src = os.path.join(os.path.dirname(oracle.__file__), "bsb_oracle_sw.c")
    so = str(tmp_path / "libsw_cf.so")
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
                           "-DORC_SW_LAZY_F_CLOSED_FORM", "-o", so, src])
    L = ctypes.CDLL(so)
    a, b, o_del, e_del, o_ins, e_ins = scoring
    jobs, seq, tags = golden_data.golden_sw_jobs(a, n=1500, seed=20261203 + 50 + o_ins)
    mat = np.ascontiguousarray(synth.fill_scmat(a, b), dtype=np.int8)
    jobs = np.ascontiguousarray(jobs)
    out = np.zeros(len(jobs), oracle.KSWR_DTYPE)
    p = ctypes.c_void_p
    L.orc_align2_batch.argtypes = [ctypes.c_int64, p, p, p] + [ctypes.c_int] * 4 + [p, ctypes.c_int]
    L.orc_align2_batch(len(jobs), jobs.ctypes.data, seq.ctypes.data, mat.ctypes.data, o_del, e_del, o_ins, e_ins,
                       out.ctypes.data, 8)
    ref = oracle.align2_batch(jobs, seq, mat, o_del, e_del, o_ins, e_ins, n_threads=8)
    for f in FIELDS:
        bad = np.nonzero(out[f] != ref[f])[0]
        assert len(bad) == 0, f"{f} differs at jobs {bad[:6]} ({tags[bad[:6]]})"
