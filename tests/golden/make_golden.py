"""Regenerate the golden fixtures in tests/golden/ from the reference itself.

Run from the repository root in a container that holds the reference
sources (this script, and only this script, reads them):

    make -f oracle/Makefile.ref -j8          # reference objects -> oracle/_ref/
    python tests/golden/make_golden.py ksw     # ksw_extend2 tuples
    python tests/golden/make_golden.py index   # reference `bwa index` checksums
    python tests/golden/make_golden.py reads   # seeds / chains / regions (before and after
                                               # mem_sort_dedup_patch) / job stream
    python tests/golden/make_golden.py cigar   # bwa_gen_cigar2 records (CIGAR, MD, XB)
    python tests/golden/make_golden.py sw      # ksw_align2 results (mate-rescue Smith-Waterman)

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

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from golden_data import (GENOME, GENOME_REP, OPTS, golden_cigar_jobs, golden_genome, golden_reads_indel,  # noqa: E402
                         golden_genome_rep, golden_reads, golden_reads_rep, golden_sw_jobs)

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


# ------------------------------------------------------------------ index

def make_index(td, tag="", genome=golden_genome, meta=GENOME):
    fa = os.path.join(td, f"ref{tag}.fa")
    synth.write_fasta(fa, genome())
    prefix = os.path.join(td, f"ref{tag}")
    subprocess.check_call([os.path.join(REF, "bwa"), "index", "-a", "bwtsw", "-p", prefix, fa],
                          stderr=subprocess.DEVNULL)
    sums = {ext: sha256(prefix + "." + ext) for ext in ("pac", "opac", "ann", "amb", "bwt", "sa")}
    import json
    fn = os.path.join(HERE, f"index{tag}_sha256.json")
    with open(fn, "w") as f:
        json.dump({"genome": meta, "files": sums}, f, indent=1)
    print(fn)
    return prefix


# ------------------------------------------------------------------ reads

def parse_dump(prefix, n_reads):
    """Parse the binary streams golden_dump writes (see oracle/golden_dump.c)."""
    out = {}
    b = open(prefix + ".smem.bin", "rb").read()
    off, smem, smem_off = 0, [], [0]
    for _ in range(n_reads):
        r, n = np.frombuffer(b, np.int32, 2, off); off += 8
        smem.append(np.frombuffer(b, np.uint64, 4 * n, off).reshape(n, 4)); off += 32 * n
        smem_off.append(smem_off[-1] + n)
    out["smem"] = np.concatenate(smem) if smem else np.zeros((0, 4), np.uint64)
    out["smem_off"] = np.array(smem_off, np.int64)
    b = open(prefix + ".chain.bin", "rb").read()
    off = 0
    seed_dt = np.dtype([("rbeg", "<i8"), ("qbeg", "<i4"), ("len", "<i4"), ("score", "<i4"), ("pad", "<i4")])
    for stage in ("chain0", "chain1"):
        out[stage + "_rows"], out[stage + "_seeds"], out[stage + "_off"] = [], [], [0]
    for _ in range(n_reads):
        for stage in ("chain0", "chain1"):
            r, n = np.frombuffer(b, np.int32, 2, off); off += 8
            for _c in range(n):
                h = np.frombuffer(b, np.int32, 5, off); off += 20
                pos = np.frombuffer(b, np.int64, 1, off)[0]; off += 8
                ns = int(h[0])
                seeds = np.frombuffer(b, seed_dt, ns, off); off += 24 * ns
                out[stage + "_rows"].append([h[0], h[1], h[2], h[3], h[4], pos, len(out[stage + "_seeds"])])
                out[stage + "_seeds"].extend(seeds.tolist())
            out[stage + "_off"].append(len(out[stage + "_rows"]))
    for stage in ("chain0", "chain1"):
        out[stage + "_rows"] = np.array(out[stage + "_rows"], np.int64).reshape(-1, 7)
        out[stage + "_seeds"] = np.array(out[stage + "_seeds"], np.int64).reshape(-1, 5)[:, :4]
        out[stage + "_off"] = np.array(out[stage + "_off"], np.int64)
    b = open(prefix + ".reg.bin", "rb").read()
    off, regs, reg_off = 0, [], [0]
    for _ in range(n_reads):
        r, n = np.frombuffer(b, np.int32, 2, off); off += 8
        for _k in range(n):
            rr = np.frombuffer(b, np.int64, 2, off); off += 16
            v = np.frombuffer(b, np.int32, 9, off); off += 36
            fr = np.frombuffer(b, np.float32, 1, off)[0]; off += 4
            regs.append(list(rr) + list(v[:8]) + [int(np.float32(fr).view(np.int32))])
        reg_off.append(len(regs))
    out["regs"] = np.array(regs, np.int64).reshape(-1, 11)
    out["reg_off"] = np.array(reg_off, np.int64)
    # after mem_sort_dedup_patch: the same columns, n_comp in place of the padding
    b = open(prefix + ".dedup.bin", "rb").read()
    off, regs, reg_off = 0, [], [0]
    for _ in range(n_reads):
        r, n = np.frombuffer(b, np.int32, 2, off); off += 8
        for _k in range(n):
            rr = np.frombuffer(b, np.int64, 2, off); off += 16
            v = np.frombuffer(b, np.int32, 9, off); off += 36
            fr = np.frombuffer(b, np.float32, 1, off)[0]; off += 4
            regs.append(list(rr) + list(v) + [int(np.float32(fr).view(np.int32))])
        reg_off.append(len(regs))
    out["dedup"] = np.array(regs, np.int64).reshape(-1, 12)
    out["dedup_off"] = np.array(reg_off, np.int64)
    b = open(prefix + ".ksw.bin", "rb").read()
    off, kh, kr, kseq, koff = 0, [], [], [], [0]
    while off < len(b):
        h = np.frombuffer(b, np.int32, 10, off); off += 40
        res = np.frombuffer(b, np.int32, 6, off); off += 24
        q = np.frombuffer(b, np.uint8, h[1], off); off += h[1]
        t = np.frombuffer(b, np.uint8, h[2], off); off += h[2]
        kh.append(h[:7]); kr.append(res); kseq.append(q); kseq.append(t)
        koff.append(koff[-1] + h[1] + h[2])
    out["ksw_hdr"] = np.array(kh, np.int32).reshape(-1, 7)
    out["ksw_out"] = np.array(kr, np.int32).reshape(-1, 6)
    out["ksw_seq"] = np.concatenate(kseq) if kseq else np.zeros(0, np.uint8)
    out["ksw_seq_off"] = np.array(koff, np.int64)
    return out


def make_reads(td, prefix, reads=None, names=("L5", "L30"), tag=""):
    reads = golden_reads() if reads is None else reads
    offs = np.zeros(len(reads) + 1, np.int64)
    offs[1:] = np.cumsum([len(r) for r in reads])
    fin = os.path.join(td, "reads.bin")
    with open(fin, "wb") as f:
        f.write(np.array([len(reads), offs[-1]], np.int64).tobytes())
        f.write(offs.tobytes())
        f.write(np.concatenate(reads).astype(np.uint8).tobytes())
    for name in names:
        o = OPTS[name]
        fo = os.path.join(td, f"opt_{name}.bin")
        np.array(o, np.int32).tofile(fo)
        outp = os.path.join(td, f"dump_{name}")
        subprocess.check_call([os.path.join(REF, "golden_dump"), "reads", prefix, fin, outp, fo])
        d = parse_dump(outp, len(reads))
        fn = os.path.join(HERE, f"reads{tag}_{name}.npz")
        np.savez_compressed(fn, reads=np.concatenate(reads), read_off=offs, opts=np.array(o, np.int32), **d)
        print(fn, os.path.getsize(fn), "smem", len(d["smem"]), "regs", len(d["regs"]), "ksw", len(d["ksw_out"]))


# ------------------------------------------------------------------ cigar

CIGAR_SCORINGS = [("default", 1, 4, 6, 1, 6, 1), ("asym", 2, 5, 5, 3, 7, 2)]


def run_ref_gen_cigar(L, mat, o_del, e_del, o_ins, e_ins, bi, jobs, qbuf, obuf):
    """The reference bwa_gen_cigar2 (bwa.c:199-351), one call per job as mem_reg2aln
    makes it (bwamem.c:1228).  Returns (records[n, 8] int32, blob, offsets)."""
    import ctypes
    libc = ctypes.CDLL(None)
    libc.free.argtypes = [ctypes.c_void_p]
    f = L.bwa_gen_cigar2
    f.restype = ctypes.POINTER(ctypes.c_uint32)
    I = ctypes.c_int
    P = ctypes.c_void_p
    f.argtypes = [P, I, I, I, I, I, ctypes.c_int64, P, P, I, P, ctypes.c_int64, ctypes.c_int64,
                  ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I), ctypes.c_int64, P,
                  ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I)]
    mat = np.ascontiguousarray(mat, np.int8)
    pac = np.ascontiguousarray(bi.pac)
    opac = np.ascontiguousarray(bi.opac)
    recs, parts, offs = [], [], [0]
    for j in jobs:
        lq = int(j["l_query"])
        q = np.ascontiguousarray(qbuf[j["qoff"]:j["qoff"] + max(lq, 0)].copy())
        oq = np.ascontiguousarray(obuf[j["ooff"]:].copy())
        v = [I(0) for _ in range(7)]
        v[2].value = -7                                       # NM: -1 is written by the callee
        ptr = f(mat.ctypes.data, o_del, e_del, o_ins, e_ins, int(j["w"]), bi.l_pac, pac.ctypes.data,
                opac.ctypes.data, lq, q.ctypes.data if len(q) else None, int(j["rb"]), int(j["re"]),
                ctypes.byref(v[0]), ctypes.byref(v[1]), ctypes.byref(v[2]), bi.crick_l,
                oq.ctypes.data if len(oq) else None, ctypes.byref(v[3]), ctypes.byref(v[4]),
                ctypes.byref(v[5]), ctypes.byref(v[6]))
        score, n_cigar, nm = v[0].value, v[1].value, v[2].value
        if not ptr:
            status, data = 1, b""
            score = 0
        else:
            words = bytes(np.ctypeslib.as_array(ptr, (max(n_cigar, 1),))[:n_cigar].tobytes())
            if nm == -1:
                status, data = 2, words
            else:
                s = ctypes.string_at(ctypes.addressof(ptr.contents) + 4 * n_cigar)
                status, data = 0, words + s + b"\0"
            libc.free(ctypes.cast(ptr, ctypes.c_void_p))
        meth = [v[k].value for k in range(3, 7)] if status == 0 else [0, 0, 0, 0]
        recs.append([score, n_cigar if status != 1 else 0, nm if status == 0 else -1] + meth + [status])
        parts.append(data)
        offs.append(offs[-1] + len(data))
    return np.array(recs, np.int32), np.frombuffer(b"".join(parts), np.uint8).copy(), np.array(offs, np.int64)


def make_cigar(td):
    import ctypes
    import oracle
    from bsbolt_gb300 import index
    prefix = make_index(td)
    bi = index.BwaIndex(prefix)
    jobs, qbuf, obuf, tags = golden_cigar_jobs(bi.pac, bi.opac, bi.l_pac, bi.crick_l)
    L = ctypes.CDLL(os.path.join(REF, "libbwaref.so"))
    for name, a, b, o_del, e_del, o_ins, e_ins in CIGAR_SCORINGS:
        mat = synth.fill_scmat(a, b)
        # jobs where the reference reads memory it never wrote are left out (the oracle
        # reports them by status)
        o, _ = oracle.gen_cigar_batch(mat, o_del, e_del, o_ins, e_ins, bi.l_pac, bi.pac, bi.opac, bi.crick_l,
                                      jobs, qbuf, obuf)
        keep = np.nonzero(o["status"] < 3)[0]
        recs, blob, boff = run_ref_gen_cigar(L, mat, o_del, e_del, o_ins, e_ins, bi, jobs[keep], qbuf, obuf)
        fn = os.path.join(HERE, f"cigar_{name}.npz")
        np.savez_compressed(fn, keep=keep, scoring=np.array([a, b, o_del, e_del, o_ins, e_ins], np.int32),
                            recs=recs, blob=blob, blob_off=boff)
        print(fn, os.path.getsize(fn), "jobs", len(keep), "of", len(jobs),
              "status", np.bincount(recs[:, 7], minlength=3))


# ------------------------------------------------------------------ sw

SW_SCORINGS = [("default", 1, 4, 6, 1, 6, 1), ("asym", 2, 5, 5, 3, 7, 2), ("wide", 1, 3, 250, 10, 200, 60)]


def make_sw():
    """The reference ksw_align2 (ksw.c:336-360), one call per job."""
    import ctypes
    L = ctypes.CDLL(os.path.join(REF, "libbwaref.so"))

    class Kswr(ctypes.Structure):
        _fields_ = [(f, ctypes.c_int) for f in ("score", "te", "qe", "score2", "te2", "tb", "qb")]
    f = L.ksw_align2
    f.restype = Kswr
    I, P = ctypes.c_int, ctypes.c_void_p
    f.argtypes = [I, P, I, P, I, P, I, I, I, I, I, P]
    for name, a, b, o_del, e_del, o_ins, e_ins in SW_SCORINGS:
        jobs, seq, tags = golden_sw_jobs(a)
        mat = np.ascontiguousarray(synth.fill_scmat(a, b))
        recs = []
        for j in jobs:
            q = np.ascontiguousarray(seq[j["qoff"]:j["qoff"] + j["qlen"]].copy())
            t = np.ascontiguousarray(seq[j["toff"]:j["toff"] + j["tlen"]].copy())
            r = f(int(j["qlen"]), q.ctypes.data if len(q) else None, int(j["tlen"]), t.ctypes.data if len(t) else None,
                  5, mat.ctypes.data, o_del, e_del, o_ins, e_ins, int(j["xtra"]), None)
            recs.append([r.score, r.te, r.qe, r.score2, r.te2, r.tb, r.qb])
        fn = os.path.join(HERE, f"sw_{name}.npz")
        np.savez_compressed(fn, scoring=np.array([a, b, o_del, e_del, o_ins, e_ins], np.int32),
                            recs=np.array(recs, np.int32))
        print(fn, os.path.getsize(fn), "jobs", len(jobs))


if __name__ == "__main__":
    what = sys.argv[1:] or ["ksw"]
    if "ksw" in what:
        make_ksw()
    if "sw" in what:
        make_sw()
    if "cigar" in what:
        with tempfile.TemporaryDirectory() as td:
            make_cigar(td)
    if "index" in what or "reads" in what:
        with tempfile.TemporaryDirectory() as td:
            prefix = make_index(td)
            if "reads" in what:
                make_reads(td, prefix)
                make_reads(td, prefix, golden_reads_indel(), ("W5",), "_indel")
            prefix = make_index(td, "_rep", golden_genome_rep, GENOME_REP)
            if "reads" in what:
                make_reads(td, prefix, golden_reads_rep(), ("L5",), "_rep")
