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
