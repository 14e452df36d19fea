"""Regenerate the golden fixtures in tests/golden/ from the reference itself.

Run from the repository root in a container that holds the reference
sources (this script, and only this script, reads them):

    make -f oracle/Makefile.ref -j8          # reference objects -> oracle/_ref/
    python tests/golden/make_golden.py ksw     # ksw_extend2 tuples
    python tests/golden/make_golden.py index   # reference `bwa index` checksums
    python tests/golden/make_golden.py reads   # seeds / chains / regions / job stream

Every output value in the fixtures comes from the reference code compiled
from BSBolt's bsbolt/External/BWA sources (oracle/_ref/golden_dump,
oracle/_ref/bwa); the inputs come from the seeded generators in
bsbolt_gb300.synth.
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from bsbolt_gb300 import synth  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(ROOT, "oracle", "_ref")

# scoring sets: (name, a, b, o_del, e_del, o_ins, e_ins, zdrop)
SCORINGS = [
    ("default", 1, 4, 6, 1, 6, 1, 100),
    ("asym", 1, 4, 5, 3, 7, 2, 100),
    ("a2", 2, 5, 8, 2, 8, 2, 50),
    ("nozdrop", 1, 4, 6, 1, 6, 1, 0),
    ("zdrop5", 1, 4, 6, 1, 6, 1, 5),
]


def edge_jobs(rng):
    """Hand-made corner cases of ksw_extend2 (ksw.c:380-479)."""
    cases = []  # (query, target, h0, w, end_bonus)

    def rnd(n, p=(0.3, 0.0, 0.2, 0.5, 0.0)):
        p = np.asarray(p, float)
        return rng.choice(5, size=n, p=p / p.sum()).astype(np.uint8)

    q = rnd(60)
    cases.append((q, np.zeros(0, np.uint8), 30, 100, 5))            # empty target
    cases.append((rnd(1), rnd(1), 1, 100, 5))                       # 1x1, h0=1
    cases.append((rnd(1), rnd(120), 19, 100, 5))                    # single query base
    cases.append((q, q.copy(), 40, 100, 5))                          # perfect match
    cases.append((q, q.copy(), 40, 0, 5))                            # w = 0
    cases.append((q, q.copy(), 40, 1, 5))                            # w = 1
    cases.append((q, q.copy(), 40, 3, 0))                            # narrow band, no bonus
    cases.append((q, q.copy(), 40, 100, 30))                         # bsbolt's -L 30
    cases.append((q, q.copy(), 1000, 100, 5))                        # huge h0
    cases.append((np.full(50, 4, np.uint8), rnd(150), 50, 100, 5))  # all-N query
    cases.append((q, np.full(150, 4, np.uint8), 50, 100, 5))        # all-N target
    cases.append((q, rnd(30), 80, 100, 5))                           # tlen < qlen
    cases.append((rnd(250), rnd(350), 60, 100, 5))                   # longest read, random
    for L in (31, 32, 33, 63, 64, 95, 96, 127, 128, 159, 160, 191, 192, 223, 224, 254, 255,
              256, 257, 300, 383, 384, 511, 512, 700):
        qq = rnd(L)
        tt = np.concatenate([qq, rnd(100)])
        cases.append((qq, tt, 25 + L % 70, 100, 5))                  # lane-tiling boundaries
        cases.append((qq, rnd(L + 100), 25 + L % 70, 100, 5))        # unrelated at the boundary
    # repeats: a periodic query against a shifted periodic target makes the band
    # shrink and grow back over stale cells
    unit = rnd(7)
    qq = np.tile(unit, 20)[:130]
    tt = np.concatenate([rnd(3), np.tile(unit, 30)[:200]])
    for h0 in (5, 19, 40, 90):
        for w in (2, 5, 20, 100):
            cases.append((qq, tt, h0, w, 5))
    # low-complexity with indels
    qq = np.tile(np.array([0, 3], np.uint8), 60)
    tt = np.concatenate([np.tile(np.array([0, 3], np.uint8), 20), np.array([2, 2, 2], np.uint8),
                         np.tile(np.array([0, 3], np.uint8), 60)])
    for h0 in (3, 20, 60):
        cases.append((qq, tt, h0, 100, 5))
        cases.append((qq, tt, h0, 7, 5))
    return cases


def pack_cases(cases):
    parts, jobs, base = [], [], 0
    for q, t, h0, w, eb in cases:
        parts += [q, t]
        jobs.append((base, base + len(q), len(q), len(t), h0, w, eb, 0))
        base += len(q) + len(t)
    return np.array(jobs, dtype=synth.JOB_DTYPE), np.concatenate(parts).astype(np.uint8)


def run_ref_ksw(jobs, seq, mat, o_del, e_del, o_ins, e_ins, zdrop):
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        hdr = np.zeros(72, np.uint8)
        hdr[0:8] = np.frombuffer(np.int64(len(jobs)).tobytes(), np.uint8)
        hdr[8:16] = np.frombuffer(np.int64(len(seq)).tobytes(), np.uint8)
        hdr[16:41] = mat.view(np.uint8)
        hdr[48:68] = np.frombuffer(np.array([o_del, e_del, o_ins, e_ins, zdrop], np.int32).tobytes(), np.uint8)
        with open(fin, "wb") as f:
            f.write(hdr.tobytes())
            f.write(jobs.tobytes())
            f.write(seq.tobytes())
        subprocess.check_call([os.path.join(REF, "golden_dump"), "ksw", fin, fout])
        return np.fromfile(fout, np.int32).reshape(-1, 6)


def make_ksw():
    rng = np.random.Generator(np.random.PCG64(77))
    for si, (name, a, b, od, ed, oi, ei, zd) in enumerate(SCORINGS):
        n_rand = 3000 if name == "default" else 600
        jobs, seq = synth.ksw_jobs(n_rand, seed=20261203 + 1 + 1000 * si)
        ej, es = pack_cases(edge_jobs(rng))
        ej = ej.copy()
        ej["qoff"] += len(seq)
        ej["toff"] += len(seq)
        jobs = np.concatenate([jobs, ej])
        seq = np.concatenate([seq, es])
        mat = synth.fill_scmat(a, b)
        out = run_ref_ksw(jobs, seq, mat, od, ed, oi, ei, zd)
        fn = os.path.join(HERE, f"ksw_{name}.npz")
        np.savez_compressed(fn, jobs=jobs.view(np.uint8).reshape(len(jobs), -1), seq=seq, mat=mat,
                            params=np.array([od, ed, oi, ei, zd], np.int32), out=out)
        print(fn, len(jobs), os.path.getsize(fn))


def sha256(fn):
    h = hashlib.sha256()
    with open(fn, "rb") as f:
        h.update(f.read())
    return h.hexdigest()


if __name__ == "__main__":
    what = sys.argv[1:] or ["ksw"]
    if "ksw" in what:
        make_ksw()
