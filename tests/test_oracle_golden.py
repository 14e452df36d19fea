"""The oracle restatement against the reference's own outputs (CPU only).

The fixtures in tests/golden/ were produced by the reference compiled from
its sources (tests/golden/make_golden.py); these tests pin the oracle to
them before the oracle is trusted as the GPU checker.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from bsbolt_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KSW_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "ksw_*.npz")))


def load_ksw(fn):
    d = np.load(fn)
    jobs = np.ascontiguousarray(d["jobs"]).view(synth.JOB_DTYPE).reshape(-1)
    return jobs, d["seq"], d["mat"], [int(x) for x in d["params"]], d["out"]


def test_fixtures_present():
    names = {os.path.basename(f) for f in KSW_FIXTURES}
    assert {"ksw_default.npz", "ksw_asym.npz", "ksw_a2.npz", "ksw_nozdrop.npz", "ksw_zdrop5.npz"} <= names


@pytest.mark.parametrize("fn", KSW_FIXTURES, ids=lambda f: os.path.basename(f))
def test_oracle_ksw_matches_reference(fn):
    jobs, seq, mat, params, ref = load_ksw(fn)
    out, cells = oracle.ksw_batch(jobs, seq, mat, *params, n_threads=4)
    bad = np.nonzero((out != ref).any(axis=1))[0]
    assert len(bad) == 0, f"{len(bad)} tuples differ, first job {bad[:5]}"
    assert (cells >= 0).all()


def test_oracle_ksw_edge_semantics():
    # empty target: nothing extends, score stays h0 (ksw.c:471-478)
    q = np.array([0, 2, 3, 3, 0], np.uint8)
    jobs = np.zeros(1, synth.JOB_DTYPE)
    jobs[0] = (0, 5, 5, 0, 17, 100, 5, 0)
    out, cells = oracle.ksw_batch(jobs, q, synth.fill_scmat(), 6, 1, 6, 1, 100)
    assert out[0].tolist() == [17, 0, 0, 0, -1, 0] and cells[0] == 0


def test_generator_is_seeded():
    a = synth.ksw_jobs(300, seed=5)
    b = synth.ksw_jobs(300, seed=5)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    jobs, seq = a
    assert jobs["qlen"].min() >= 10 and jobs["qlen"].max() <= 140
    assert (jobs["qoff"] + jobs["qlen"] <= len(seq)).all() and (jobs["toff"] + jobs["tlen"] <= len(seq)).all()


@pytest.mark.skipif(not oracle.have_reference_ksw(), reason="reference sources not staged (oracle/_ref)")
@pytest.mark.parametrize("fn", KSW_FIXTURES, ids=lambda f: os.path.basename(f))
def test_reference_ksw_harness_reproduces_fixtures(fn):
    """The threaded harness around the reference's own ksw_extend2 (the CPU baseline of the
    extension bench) returns the fixtures' tuples: it runs the reference unchanged."""
    jobs, seq, mat, params, ref = load_ksw(fn)
    assert np.array_equal(oracle.ref_ksw_batch(jobs, seq, mat, *params, n_threads=4), ref)
