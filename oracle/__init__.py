"""CPU oracle for the bisulfite seed/extend path -- TEST INFRASTRUCTURE ONLY.

The oracle is a plain-C restatement (``bsb_oracle.c``) of the reference
algorithms in BSBolt's BWA fork (``bsbolt/External/BWA``: ``ksw.c``,
``bwt.c``, ``bwamem.c``).  Only the tests, ``__graft_entry__.smoke()`` and
the CPU-baseline legs of ``bench.py`` load it, always as the checker or the
timed CPU reference, never as the product path.  Its parity with the
reference is pinned by ``tests/golden/`` (fixtures produced by the reference
itself, compiled from its sources by ``oracle/Makefile.ref``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "liborc.so")
_lib = None


_SRC = ("bsb_oracle.c", "bsb_oracle_chain.c", "bsb_oracle_cigar.c", "bsb_oracle_sw.c", "bsb_oracle_dedup.c")
_HDR = ("bsb_oracle.h", "bsb_oracle_chain.h", "bsb_oracle_cigar.h", "bsb_oracle_sw.h", "bsb_oracle_dedup.h")


def build(force: bool = False) -> str:
    """Compile the oracle restatement into oracle/_build/liborc.so (gcc -O2)."""
    deps = [os.path.join(_HERE, f) for f in _SRC + _HDR]
    if not force and os.path.exists(_SO) and all(os.path.getmtime(_SO) >= os.path.getmtime(d) for d in deps):
        return _SO
    os.makedirs(os.path.dirname(_SO), exist_ok=True)
    tmp = _SO + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-o", tmp]
                          + [os.path.join(_HERE, f) for f in _SRC] + ["-lm"])
    os.replace(tmp, _SO)
    return _SO


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_SO):
            build()
        L = ctypes.CDLL(_SO)
        P = ctypes.c_void_p
        L.orc_ksw_batch.restype = ctypes.c_int64
        L.orc_ksw_batch.argtypes = [ctypes.c_int64, P, P, P, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int]
        L.orc_bwt_init.restype = None
        L.orc_bwt_init.argtypes = [P, ctypes.c_uint64, P, P, ctypes.c_uint64, P,
                                   ctypes.c_uint64, ctypes.c_int]
        L.orc_collect_intv_batch.restype = ctypes.c_int
        L.orc_collect_intv_batch.argtypes = [P, P, ctypes.c_int, P, P, P, ctypes.c_int64, P,
                                             ctypes.c_int]
        L.orc_bwt_sa_batch.restype = None
        L.orc_align2_batch.restype = None
        L.orc_align2_batch.argtypes = [ctypes.c_int64, P, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, P, ctypes.c_int]
        L.orc_gen_cigar_batch.restype = ctypes.c_int64
        L.orc_gen_cigar_batch.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int64, P, P, ctypes.c_int64, ctypes.c_int64, P, P, P, P, P,
                                          ctypes.c_int64, ctypes.c_int]
        L.orc_bwt_sa_batch.argtypes = [P, ctypes.c_int64, P, P, ctypes.c_int]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def ksw_batch(jobs: np.ndarray, seq: np.ndarray, mat: np.ndarray, o_del: int, e_del: int,
              o_ins: int, e_ins: int, zdrop: int, n_threads: int = 1):
    """Reference ksw_extend2 (ksw.c:380-479) over a job table.

    Returns (out[n,6] int32, cells[n] int64)."""
    jobs = np.ascontiguousarray(jobs)
    seq = np.ascontiguousarray(seq, dtype=np.uint8)
    mat = np.ascontiguousarray(mat, dtype=np.int8)
    n = len(jobs)
    out = np.zeros((n, 6), np.int32)
    cells = np.zeros(n, np.int64)
    lib().orc_ksw_batch(n, _p(jobs), _p(seq), _p(mat), o_del, e_del, o_ins, e_ins, zdrop,
                        _p(out), _p(cells), n_threads)
    return out, cells


_REF_KSW = os.path.join(_HERE, "_ref", "libref_ksw.so")


def have_reference_ksw() -> bool:
    """Whether the reference's own ksw_extend2 was built here (oracle/Makefile.ref, from the
    staged reference sources)."""
    return os.path.exists(_REF_KSW)


def ref_ksw_batch(jobs: np.ndarray, seq: np.ndarray, mat: np.ndarray, o_del: int, e_del: int,
                  o_ins: int, e_ins: int, zdrop: int, n_threads: int = 1) -> np.ndarray:
    """The reference's compiled ksw_extend2 (ksw.c:380-479, linked from its sources into
    oracle/_ref/libref_ksw.so by oracle/ref_ksw_batch.c) over a job table on n_threads host
    threads.  Returns out[n,6] int32."""
    L = ctypes.CDLL(_REF_KSW)
    P = ctypes.c_void_p
    L.ref_ksw_batch.restype = ctypes.c_int
    L.ref_ksw_batch.argtypes = [ctypes.c_int64, P, P, P] + [ctypes.c_int] * 5 + [P, ctypes.c_int]
    jobs = np.ascontiguousarray(jobs)
    seq = np.ascontiguousarray(seq, dtype=np.uint8)
    mat = np.ascontiguousarray(mat, dtype=np.int8)
    out = np.zeros((len(jobs), 6), np.int32)
    L.ref_ksw_batch(len(jobs), _p(jobs), _p(seq), _p(mat), o_del, e_del, o_ins, e_ins, zdrop, _p(out), n_threads)
    return out


class OracleBwt:
    """The FM-index as the oracle sees it (bwt.h:46-58)."""

    def __init__(self, primary, L2, bwt_words: np.ndarray, sa: np.ndarray, sa_intv: int):
        self.bwt_words = np.ascontiguousarray(bwt_words, dtype=np.uint32)
        self.sa = np.ascontiguousarray(sa, dtype=np.uint64)
        self.L2 = np.ascontiguousarray(np.asarray(L2, dtype=np.uint64)[-4:])
        self._struct = (ctypes.c_uint8 * 256)()
        lib().orc_bwt_init(ctypes.addressof(self._struct), int(primary), _p(self.L2),
                           _p(self.bwt_words), len(self.bwt_words), _p(self.sa), len(self.sa),
                           int(sa_intv))

    @property
    def ptr(self):
        return ctypes.c_void_p(ctypes.addressof(self._struct))

    def collect_intv(self, seqs: np.ndarray, offs: np.ndarray, min_seed_len=19, split_factor=1.5,
                     split_width=10, max_mem_intv=20, n_threads=1):
        """mem_collect_intv (bwamem.c:118-166) for every read. Returns (intv[m,4] u64, off[n+1])."""
        class _Opt(ctypes.Structure):
            _fields_ = [("min_seed_len", ctypes.c_int), ("split_factor", ctypes.c_float),
                        ("split_width", ctypes.c_int), ("max_mem_intv", ctypes.c_int)]
        opt = _Opt(min_seed_len, split_factor, split_width, max_mem_intv)
        seqs = np.ascontiguousarray(seqs, dtype=np.uint8)
        offs = np.ascontiguousarray(offs, dtype=np.int64)
        n = len(offs) - 1
        cap = int((offs[1:] - offs[:-1]).sum()) * 4 + 16 * max(n, 1)
        out = np.zeros((cap, 4), np.uint64)
        out_off = np.zeros(n + 1, np.int64)
        rc = lib().orc_collect_intv_batch(self.ptr, ctypes.byref(opt), n, _p(seqs), _p(offs),
                                          _p(out), cap, _p(out_off), n_threads)
        if rc != 0:
            raise RuntimeError("oracle collect_intv overflow")
        return out[: out_off[-1]].copy(), out_off

    def sa_lookup(self, k: np.ndarray, n_threads=1):
        """bwt_sa (bwt.c:86-96) for every row in k."""
        k = np.ascontiguousarray(k, dtype=np.uint64)
        pos = np.zeros(len(k), np.uint64)
        lib().orc_bwt_sa_batch(self.ptr, len(k), _p(k), _p(pos), n_threads)
        return pos


# ---------------------------------------------------------------- chaining / extension

CHAIN_DTYPE = np.dtype([("n", "<i4"), ("rid", "<i4"), ("first", "<i4"), ("kept", "<i4"), ("w", "<i4"),
                        ("is_alt", "<i4"), ("frac_rep", "<f4"), ("seed_off", "<i4"), ("pos", "<i8")])
SEED_DTYPE = np.dtype([("rbeg", "<i8"), ("qbeg", "<i4"), ("len", "<i4"), ("score", "<i4"), ("pad", "<i4")])
REG_DTYPE = np.dtype([("rb", "<i8"), ("re", "<i8"), ("qb", "<i4"), ("qe", "<i4"), ("rid", "<i4"),
                      ("score", "<i4"), ("truesc", "<i4"), ("w", "<i4"), ("seedcov", "<i4"),
                      ("seedlen0", "<i4"), ("frac_rep", "<f4"), ("n_comp", "<i4")])
ANN_DTYPE = np.dtype([("offset", "<i8"), ("len", "<i4"), ("is_alt", "<i4")])


class Opt(ctypes.Structure):
    """orc_opt_t: the mem_opt_t fields of the path (BWA defaults, bwamem.c:50-88)."""
    _fields_ = [(f, ctypes.c_int32) for f in ("a", "b", "o_del", "e_del", "o_ins", "e_ins", "w", "zdrop",
                                               "pen_clip5", "pen_clip3", "min_seed_len", "max_occ",
                                               "max_chain_gap", "min_chain_weight", "max_chain_extend")] + \
               [("mask_level", ctypes.c_float), ("drop_ratio", ctypes.c_float), ("split_factor", ctypes.c_float),
                ("split_width", ctypes.c_int32), ("max_mem_intv", ctypes.c_int32),
                ("mat", ctypes.c_int8 * 25), ("pad_", ctypes.c_int8 * 3), ("mask_level_redun", ctypes.c_float)]

    @classmethod
    def from_list(cls, o):
        """From [a, b, o_del, e_del, o_ins, e_ins, w, zdrop, pen_clip5, pen_clip3,
        min_seed_len, max_occ, split_width, max_mem_intv, max_chain_gap]."""
        o = [int(x) for x in o]
        opt = cls(a=o[0], b=o[1], o_del=o[2], e_del=o[3], o_ins=o[4], e_ins=o[5], w=o[6], zdrop=o[7],
                  pen_clip5=o[8], pen_clip3=o[9], min_seed_len=o[10], max_occ=o[11], max_chain_gap=o[14],
                  min_chain_weight=0, max_chain_extend=1 << 30, mask_level=0.5, drop_ratio=0.5,
                  split_factor=1.5, split_width=o[12], max_mem_intv=o[13], mask_level_redun=0.95)
        for i in range(4):
            for j in range(4):
                opt.mat[i * 5 + j] = o[0] if i == j else -o[1]
        for k in range(25):
            if k % 5 == 4 or k >= 20:
                opt.mat[k] = -1
        return opt


class _Bns(ctypes.Structure):
    _fields_ = [("l_pac", ctypes.c_int64), ("n_seqs", ctypes.c_int32), ("anns", ctypes.c_void_p),
                ("pac", ctypes.c_void_p)]


class _AlignOut(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("chain0", "chain0_off", "seeds0", "seeds0_off", "chain1",
                                              "chain1_off", "regs", "regs_off")] + [("cells", ctypes.c_int64)]


def align_regs(obwt: "OracleBwt", anns: np.ndarray, pac: np.ndarray, l_pac: int, opt: Opt,
               seqs: np.ndarray, offs: np.ndarray, n_threads: int = 1):
    """Seeds -> chains -> filter -> mem_chain2aln per read (bwamem.c:1157-1180, before dedup).

    Returns a dict of numpy arrays: chain0/seeds0 (mem_chain output in tree order),
    chain1 (after mem_chain_flt), regs (pre-dedup regions), each with *_off[n+1]."""
    L = lib()
    L.orc_align_regs_batch.restype = ctypes.c_int
    L.orc_align_regs_batch.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                                               ctypes.c_void_p, ctypes.c_int]
    L.orc_align_out_free.argtypes = [ctypes.c_void_p]
    anns = np.ascontiguousarray(anns, dtype=ANN_DTYPE)
    pac = np.ascontiguousarray(pac, dtype=np.uint8)
    bns = _Bns(l_pac, len(anns), anns.ctypes.data, pac.ctypes.data)
    seqs = np.ascontiguousarray(seqs, dtype=np.uint8)
    offs = np.ascontiguousarray(offs, dtype=np.int64)
    n = len(offs) - 1
    out = _AlignOut()
    rc = L.orc_align_regs_batch(obwt.ptr, ctypes.byref(bns), ctypes.byref(opt), n, _p(seqs), _p(offs),
                                ctypes.byref(out), n_threads)
    res = {}
    for name, dt in (("chain0", CHAIN_DTYPE), ("seeds0", SEED_DTYPE), ("chain1", CHAIN_DTYPE), ("regs", REG_DTYPE)):
        off = np.ctypeslib.as_array(ctypes.cast(getattr(out, name + "_off"), ctypes.POINTER(ctypes.c_int64)),
                                    (n + 1,)).copy()
        cnt = int(off[-1])
        buf = ctypes.string_at(getattr(out, name), cnt * dt.itemsize) if cnt else b""
        res[name] = np.frombuffer(buf, dt).copy()
        res[name + "_off"] = off
    res["cells"] = int(out.cells)
    L.orc_align_out_free(ctypes.byref(out))
    if rc != 0:
        raise RuntimeError(f"oracle align_regs failed ({rc})")
    return res


CIGAR_OUT_DTYPE = np.dtype([("score", "<i4"), ("n_cigar", "<i4"), ("NM", "<i4"), ("cg_meth", "<i4"),
                            ("cg_unmeth", "<i4"), ("ch_meth", "<i4"), ("ch_unmeth", "<i4"), ("status", "<i4"),
                            ("off", "<i8"), ("bytes", "<i4"), ("pad", "<i4")])


def gen_cigar_batch(mat, o_del, e_del, o_ins, e_ins, l_pac, pac, opac, crick_l, jobs, qbuf, obuf,
                    n_threads: int = 1):
    """Reference bwa_gen_cigar2 (bwa.c:199-351) over a job table, as mem_reg2aln calls it.

    Returns (out[CIGAR_OUT_DTYPE], blob uint8): for status 0 a job's bytes are its
    CIGAR words then the NUL-terminated "MD\tXB:Z:calls" string; status 2 has the
    words only."""
    mat = np.ascontiguousarray(mat, dtype=np.int8)
    pac = np.ascontiguousarray(pac, dtype=np.uint8)
    opac = np.ascontiguousarray(opac, dtype=np.uint8)
    jobs = np.ascontiguousarray(jobs)
    qbuf = np.ascontiguousarray(qbuf, dtype=np.uint8)
    obuf = np.ascontiguousarray(obuf, dtype=np.uint8)
    n = len(jobs)
    out = np.zeros(n, CIGAR_OUT_DTYPE)
    cap = int(np.maximum(jobs["l_query"], 0).sum() + np.maximum(jobs["re"] - jobs["rb"], 0).clip(0, 1 << 20).sum()) * 16 + 64 * n + 64
    blob = np.zeros(cap, np.uint8)
    used = lib().orc_gen_cigar_batch(_p(mat), o_del, e_del, o_ins, e_ins, l_pac, _p(pac), _p(opac), crick_l, n,
                                     _p(jobs), _p(qbuf) if len(qbuf) else None, _p(obuf) if len(obuf) else None,
                                     _p(out), _p(blob), cap, n_threads)
    if used < 0:
        raise RuntimeError("oracle CIGAR blob too small")
    return out, blob[:used].copy()


SW_JOB_DTYPE = np.dtype([("qoff", "<i8"), ("toff", "<i8"), ("qlen", "<i4"), ("tlen", "<i4"), ("xtra", "<i4"),
                         ("pad", "<i4")])
KSWR_DTYPE = np.dtype([("score", "<i4"), ("te", "<i4"), ("qe", "<i4"), ("score2", "<i4"), ("te2", "<i4"),
                       ("tb", "<i4"), ("qb", "<i4")])
KSW_XBYTE, KSW_XSTOP, KSW_XSUBO, KSW_XSTART = 0x10000, 0x20000, 0x40000, 0x80000


def align2_batch(jobs, seq, mat, o_del, e_del, o_ins, e_ins, n_threads: int = 1):
    """Reference ksw_align2 (ksw.c:336-360) over a job table (SW_JOB_DTYPE).  Returns kswr_t records."""
    jobs = np.ascontiguousarray(jobs, dtype=SW_JOB_DTYPE)
    seq = np.ascontiguousarray(seq, dtype=np.uint8)
    mat = np.ascontiguousarray(mat, dtype=np.int8)
    out = np.zeros(len(jobs), KSWR_DTYPE)
    lib().orc_align2_batch(len(jobs), _p(jobs), _p(seq), _p(mat), o_del, e_del, o_ins, e_ins, _p(out), n_threads)
    return out


def sort_dedup_batch(opt, l_pac, pac, seqs, offs, regs, regs_off):
    """mem_sort_dedup_patch (bwamem.c:441-493) per read on pre-dedup regions (REG_DTYPE, per
    read regs[regs_off[r]:regs_off[r+1]]); reads are nt4 seqs[offs[r]:offs[r+1]].
    Returns (regions after dedup, their offsets)."""
    L = lib()
    L.orc_sort_dedup_batch.restype = None
    L.orc_sort_dedup_batch.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int] + \
        [ctypes.c_void_p] * 6
    pac = np.ascontiguousarray(pac, dtype=np.uint8)
    seqs = np.ascontiguousarray(seqs, dtype=np.uint8)
    offs = np.ascontiguousarray(offs, dtype=np.int64)
    regs = np.ascontiguousarray(regs, dtype=REG_DTYPE)
    regs_off = np.ascontiguousarray(regs_off, dtype=np.int64)
    n = len(offs) - 1
    out = np.zeros(max(len(regs), 1), REG_DTYPE)
    out_off = np.zeros(n + 1, np.int64)
    L.orc_sort_dedup_batch(ctypes.byref(opt), l_pac, _p(pac), n, _p(seqs), _p(offs), _p(regs), _p(regs_off), _p(out),
                           _p(out_off))
    return out[:int(out_off[-1])].copy(), out_off


def regs_from_golden(rows):
    """REG_DTYPE records from the fixtures' region rows (rb, re, qb, qe, rid, score, truesc,
    w, seedcov, seedlen0, [n_comp,] frac_rep bits)."""
    rows = np.asarray(rows, np.int64)
    r = np.zeros(len(rows), REG_DTYPE)
    for i, f in enumerate(["rb", "re", "qb", "qe", "rid", "score", "truesc", "w", "seedcov", "seedlen0"]):
        r[f] = rows[:, i]
    if rows.shape[1] == 12:
        r["n_comp"] = rows[:, 10]
    r["frac_rep"] = rows[:, -1].astype(np.int32).view(np.float32)
    return r
