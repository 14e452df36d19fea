"""CIGAR / MD / XB oracle against the reference's own bwa_gen_cigar2 (CPU only).

* the oracle restatement of bwa_gen_cigar2 + ksw_global2 reproduces every record
  the reference produced (tests/golden/cigar_*.npz: score, CIGAR words, NM, the
  MD and XB strings, the four methylation counts, reject / no-MD outcomes) for
  reads on both strands of Watson and Crick contigs, two scoring sets;
* jobs whose 2-base context window is clipped at an end of the doubled sequence
  (where the reference reads past its buffer) are reported with status 3.
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


@pytest.fixture(scope="module")
def bi(tmp_path_factory):
    d = tmp_path_factory.mktemp("cigidx")
    fa = str(d / "ref.fa")
    synth.write_fasta(fa, golden_data.golden_genome())
    prefix = str(d / "ref")
    index.build_index(fa, prefix)
    return index.BwaIndex(prefix)


def split_records(out, blob):
    return [bytes(blob[o["off"]:o["off"] + o["bytes"]]) for o in out]


@pytest.mark.parametrize("name", ["default", "asym"])
def test_oracle_gen_cigar_matches_reference(bi, name):
    g = np.load(os.path.join(GOLDEN, f"cigar_{name}.npz"))
    a, b, o_del, e_del, o_ins, e_ins = (int(v) for v in g["scoring"])
    jobs, qbuf, obuf, tags = golden_data.golden_cigar_jobs(bi.pac, bi.opac, bi.l_pac, bi.crick_l)
    out, blob = oracle.gen_cigar_batch(synth.fill_scmat(a, b), o_del, e_del, o_ins, e_ins, bi.l_pac, bi.pac,
                                       bi.opac, bi.crick_l, jobs, qbuf, obuf, n_threads=4)
    keep = g["keep"]
    rec = g["recs"]
    o = out[keep]
    for i, f in enumerate(("score", "n_cigar", "NM", "cg_meth", "cg_unmeth", "ch_meth", "ch_unmeth", "status")):
        bad = np.nonzero(o[f] != rec[:, i])[0]
        assert len(bad) == 0, f"{f} differs for jobs {keep[bad[:5]]} ({tags[keep[bad[:5]]]})"
    got = split_records(o, blob)
    for k, j in enumerate(keep):
        want = bytes(g["blob"][g["blob_off"][k]:g["blob_off"][k + 1]])
        assert got[k] == want, f"job {j} ({tags[j]}): {got[k]!r} != {want!r}"
    # every kind of job is represented, and every status the reference can give
    assert set(np.unique(rec[:, 7])) == {0, 1, 2}
    assert (o["n_cigar"][o["status"] == 0] > 1).sum() > 50            # gapped CIGARs
    assert sum(b"^" in r for r in got) > 5                             # deletions in MD


def test_oracle_gen_cigar_clipped_windows(bi):
    jobs, qbuf, obuf, tags = golden_data.golden_cigar_jobs(bi.pac, bi.opac, bi.l_pac, bi.crick_l)
    out, _ = oracle.gen_cigar_batch(synth.fill_scmat(1, 4), 6, 1, 6, 1, bi.l_pac, bi.pac, bi.opac, bi.crick_l,
                                    jobs, qbuf, obuf)
    clipped = np.array([t.startswith("clipped") for t in tags])
    assert (out["status"][clipped] == 3).all()
    assert (out["status"][~clipped] != 3).all()
    assert (out["bytes"][clipped] == 0).all()


def test_oracle_ksw_global2_small_cases():
    """ksw_global2 (ksw.c:504-606) on hand-checked cases: identity, one mismatch,
    one insertion, one deletion (leftmost placement after the strand flip is the
    caller's job; here the plain forward case)."""
    mat = synth.fill_scmat(1, 4)
    L = oracle.lib()
    import ctypes

    def glob(q, t, w):
        q = np.asarray(q, np.uint8)
        t = np.asarray(t, np.uint8)
        cig = np.zeros(len(q) + len(t) + 2, np.uint32)
        n = ctypes.c_int(0)
        ex = ctypes.c_int(0)
        L.orc_ksw_global2.restype = ctypes.c_int
        I, P = ctypes.c_int, ctypes.c_void_p
        L.orc_ksw_global2.argtypes = [I, P, I, P, P, I, I, I, I, I, ctypes.POINTER(I), P, ctypes.POINTER(I)]
        sc = L.orc_ksw_global2(len(q), q.ctypes.data, len(t), t.ctypes.data, mat.ctypes.data, 6, 1, 6, 1, w,
                               ctypes.byref(n), cig.ctypes.data, ctypes.byref(ex))
        ops = [(int(c) >> 4, "MID"[int(c) & 0xf]) for c in cig[:n.value]]
        return sc, ops, ex.value

    s = [0, 1, 2, 3] * 10
    assert glob(s, s, 5) == (40, [(40, "M")], 0)
    m = list(s)
    m[17] = (m[17] + 1) % 4
    assert glob(m, s, 5) == (35, [(40, "M")], 0)
    ins = s[:20] + [3, 3] + s[20:]
    sc, ops, ex = glob(ins, s, 5)
    assert ex == 0 and sc == 40 - 6 - 2 and [op for _, op in ops] == ["M", "I", "M"] and sum(n for n, o in ops if o == "I") == 2
    dele = s[:20] + s[23:]
    sc, ops, ex = glob(dele, s, 5)
    assert ex == 0 and sc == 37 - 6 - 3 and [op for _, op in ops] == ["M", "D", "M"] and sum(n for n, o in ops if o == "D") == 3
