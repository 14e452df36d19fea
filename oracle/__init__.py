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


def build(force: bool = False) -> str:
    """Compile the oracle restatement into oracle/_build/liborc.so (gcc -O2)."""
    src = os.path.join(_HERE, "bsb_oracle.c")
    if (not force and os.path.exists(_SO)
            and os.path.getmtime(_SO) >= os.path.getmtime(src)
            and os.path.getmtime(_SO) >= os.path.getmtime(os.path.join(_HERE, "bsb_oracle.h"))):
        return _SO
    os.makedirs(os.path.dirname(_SO), exist_ok=True)
    tmp = _SO + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-pthread", "-o", tmp, src])
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
