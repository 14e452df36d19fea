"""The SSE2 stand-in (bsbolt_gb300/integration/compat/emmintrin.h) runs BWA's striped
Smith-Waterman exactly as the real SSE2 build does.

BWA's ksw.c, built against the stand-in (oracle/_ref/libksw_compat.so: scalar lanes on
x86-64, NEON on the Arm host of a GB300 node), must return every kswr_t field that the
reference's own SSE2 build returned for tests/golden/sw_*.npz (three scoring sets, byte
and word lanes, saturation, suboptimal hits, start positions), and every ksw_extend2
tuple of tests/golden/ksw_*.npz.  This is what lets the stock `bwa` and `bwa_gpu` build on
the Arm host with the reference's results.  CPU only; skipped where the reference
sources were not staged.
"""
import ctypes
import os
import sys

import numpy as np
import pytest

from bsbolt_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
LIB = os.path.join(ROOT, "oracle", "_ref", "libksw_compat.so")
sys.path.insert(0, GOLDEN)
import golden_data  # noqa: E402

pytestmark = pytest.mark.skipif(not os.path.exists(LIB), reason="reference sources not staged (oracle/_ref)")


class Kswr(ctypes.Structure):
    _fields_ = [(f, ctypes.c_int) for f in ("score", "te", "qe", "score2", "te2", "tb", "qb")]


@pytest.fixture(scope="module")
def lib():
    L = ctypes.CDLL(LIB)
    I, P = ctypes.c_int, ctypes.c_void_p
    L.ksw_align2.restype = Kswr
    L.ksw_align2.argtypes = [I, P, I, P, I, P, I, I, I, I, I, P]
    L.ksw_extend2.restype = I
    L.ksw_extend2.argtypes = [I, P, I, P, I, P, I, I, I, I, I, I, I, I] + [ctypes.POINTER(I)] * 5
    return L


@pytest.mark.parametrize("name", ["default", "asym", "wide"])
def test_compat_ksw_align2_matches_sse2_reference(lib, name):
    g = np.load(os.path.join(GOLDEN, f"sw_{name}.npz"))
    a, b, o_del, e_del, o_ins, e_ins = (int(v) for v in g["scoring"])
    jobs, seq, tags = golden_data.golden_sw_jobs(a)
    mat = np.ascontiguousarray(synth.fill_scmat(a, b), dtype=np.int8)
    got = []
    for j in jobs:
        q = np.ascontiguousarray(seq[j["qoff"]:j["qoff"] + j["qlen"]])
        t = np.ascontiguousarray(seq[j["toff"]:j["toff"] + j["tlen"]])
        r = lib.ksw_align2(int(j["qlen"]), q.ctypes.data if len(q) else None, int(j["tlen"]),
                           t.ctypes.data if len(t) else None, 5, mat.ctypes.data, o_del, e_del, o_ins, e_ins,
                           int(j["xtra"]), None)
        got.append([r.score, r.te, r.qe, r.score2, r.te2, r.tb, r.qb])
    got = np.array(got, np.int32)
    bad = np.nonzero((got != g["recs"]).any(axis=1))[0]
    assert len(bad) == 0, f"jobs {bad[:6]} ({tags[bad[:6]]}): {got[bad[:3]]} vs {g['recs'][bad[:3]]}"


@pytest.mark.parametrize("fn", ["ksw_default.npz", "ksw_asym.npz"])
def test_compat_ksw_extend2_matches_reference(lib, fn):
    g = np.load(os.path.join(GOLDEN, fn))
    jobs = np.ascontiguousarray(g["jobs"]).view(synth.JOB_DTYPE).reshape(-1)
    seq, out = g["seq"], g["out"]
    mat = np.ascontiguousarray(g["mat"], dtype=np.int8)
    o_del, e_del, o_ins, e_ins, zdrop = (int(v) for v in g["params"])
    v = [ctypes.c_int() for _ in range(5)]
    n = min(len(jobs), 3000)
    got = np.zeros((n, 6), np.int32)
    for i in range(n):
        j = jobs[i]
        q = np.ascontiguousarray(seq[j["qoff"]:j["qoff"] + j["qlen"]])
        t = np.ascontiguousarray(seq[j["toff"]:j["toff"] + j["tlen"]])
        got[i, 0] = lib.ksw_extend2(int(j["qlen"]), q.ctypes.data if len(q) else None, int(j["tlen"]),
                                    t.ctypes.data if len(t) else None, 5, mat.ctypes.data, o_del, e_del, o_ins,
                                    e_ins, int(j["w"]), int(j["end_bonus"]), zdrop, int(j["h0"]),
                                    *[ctypes.byref(x) for x in v])
        got[i, 1:] = [x.value for x in v]
    assert np.array_equal(got, out[:n])
