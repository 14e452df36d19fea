"""FM-index files in BWA's formats: build (host C, SA-IS; or the suffix array on the GPU) and load.

``build_index(fasta, prefix)`` writes <prefix>.{pac,opac,ann,amb,bwt,sa} exactly
as BSBolt's ``bwa index -a bwtsw`` does (bsbolt/External/BWA/bwtindex.c:256-321);
``build_index(fasta, prefix, ctx=ctx)`` sorts the suffixes on the GPU
(bsb_build_bwt: prefix doubling with 64-bit ranks in chunks that fit device memory,
where the host SA-IS stops at 2^31 symbols), which returns the BWT and the sampled
suffix array, and writes the same files.
``BwaIndex(prefix)`` reads them back into numpy arrays (bwt_restore_bwt,
bwt_restore_sa, bns_restore: bwt.c:420-457, bntseq.c:99-176).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_host = None


def host_lib():
    global _host
    if _host is None:
        if not os.path.exists(_build.LIB_HOST):
            raise RuntimeError(f"{_build.LIB_HOST} is missing: run __graft_entry__.build()")
        L = ctypes.CDLL(_build.LIB_HOST)
        L.bsbh_index_fasta.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        L.bsbh_index_fasta.restype = ctypes.c_int
        L.bsbh_suffix_array.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
        L.bsbh_suffix_array.restype = ctypes.c_int
        L.bsbh_index_fasta_nobwt.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64)]
        L.bsbh_index_fasta_nobwt.restype = ctypes.c_int
        L.bsbh_write_bwt_sa64.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                          ctypes.c_int]
        L.bsbh_write_bwt_sa64.restype = ctypes.c_int
        L.bsbh_write_bwt_packed.argtypes = [ctypes.c_char_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_uint64,
                                            ctypes.c_void_p, ctypes.c_int]
        L.bsbh_write_bwt_packed.restype = ctypes.c_int
        _host = L
    return _host


def build_index(fasta: str, prefix: str, ctx=None, chunk: int = 0, sa_intv: int = 32):
    """<prefix>.{pac,opac,ann,amb,bwt,sa} of a FASTA file; with ctx (an extend.Context) the
    suffixes are sorted on that GPU (bsb_build_bwt; chunk > 0 caps the suffixes one device sort
    takes, 0 lets the free device memory decide) and the seconds of each step are returned:
    reading and packing the FASTA, the GPU sort with its copies, writing .bwt/.sa."""
    import time
    if ctx is None:
        rc = host_lib().bsbh_index_fasta(fasta.encode(), prefix.encode())
        if rc != 0:
            raise RuntimeError(f"index build failed ({rc}) for {fasta}")
        return None
    from . import _lib
    t0 = time.perf_counter()
    l_pac = ctypes.c_int64()
    rc = host_lib().bsbh_index_fasta_nobwt(fasta.encode(), prefix.encode(), ctypes.byref(l_pac))
    if rc != 0:
        raise RuntimeError(f"index build failed ({rc}) for {fasta}")
    n = l_pac.value
    pac = np.fromfile(prefix + ".pac", dtype=np.uint8)[: (n + 3) // 4].copy()
    bwt = np.empty((2 * n + 15) // 16, np.uint32)
    sa = np.empty((2 * n + sa_intv) // sa_intv, np.uint64)
    primary = ctypes.c_uint64()
    t1 = time.perf_counter()
    _lib.check(ctx.handle, ctx.L.bsb_build_bwt(ctx.handle, pac.ctypes.data_as(ctypes.c_void_p), n, sa_intv, chunk,
                                               bwt.ctypes.data_as(ctypes.c_void_p), ctypes.byref(primary),
                                               sa.ctypes.data_as(ctypes.c_void_p)))
    t2 = time.perf_counter()
    rc = host_lib().bsbh_write_bwt_packed(prefix.encode(), 2 * n, bwt.ctypes.data_as(ctypes.c_void_p),
                                          primary.value, sa.ctypes.data_as(ctypes.c_void_p), sa_intv)
    if rc != 0:
        raise RuntimeError(f"writing {prefix}.bwt/.sa failed ({rc})")
    return {"text_symbols": 2 * n, "pack_s": round(t1 - t0, 1), "gpu_sort_s": round(t2 - t1, 1),
            "write_s": round(time.perf_counter() - t2, 1)}


def suffix_array(text: np.ndarray) -> np.ndarray:
    """SA of text+'$' (text = nt4 codes 0..3), n+1 entries; SA[0] = n."""
    text = np.ascontiguousarray(text, dtype=np.uint8)
    sa = np.zeros(len(text) + 1, np.int32)
    rc = host_lib().bsbh_suffix_array(ctypes.c_void_p(text.ctypes.data), len(text),
                                      ctypes.c_void_p(sa.ctypes.data))
    if rc != 0:
        raise RuntimeError("suffix array construction failed")
    return sa


class Ann:
    __slots__ = ("name", "anno", "offset", "len", "n_ambs", "is_crick")

    def __init__(self, name, anno, offset, length, n_ambs):
        self.is_crick = "_crick_bs" in name
        self.name = name[:-9] if self.is_crick else name     # formatCrickRname (bs_helpers.cpp:74-76)
        self.anno, self.offset, self.len, self.n_ambs = anno, offset, length, n_ambs


class BwaIndex:
    """The arrays of a bisulfite BWA index, as the reference holds them in memory."""

    def __init__(self, prefix: str):
        self.prefix = prefix
        with open(prefix + ".bwt", "rb") as f:
            hdr = np.frombuffer(f.read(40), np.uint64)
            self.primary = int(hdr[0])
            self.L2 = np.concatenate([[0], hdr[1:5]]).astype(np.uint64)
            self.bwt = np.frombuffer(f.read(), np.uint32).copy()
        self.seq_len = int(self.L2[4])
        with open(prefix + ".sa", "rb") as f:
            hdr = np.frombuffer(f.read(56), np.uint64)
            if int(hdr[0]) != self.primary or int(hdr[6]) != self.seq_len:
                raise ValueError("SA-BWT inconsistency")
            self.sa_intv = int(hdr[5])
            rest = np.frombuffer(f.read(), np.uint64)
        self.sa = np.concatenate([np.array([np.iinfo(np.uint64).max], np.uint64), rest])
        self.n_sa = (self.seq_len + self.sa_intv) // self.sa_intv
        if len(self.sa) != self.n_sa:
            raise ValueError("short .sa file")
        with open(prefix + ".ann") as f:
            first = f.readline().split()
            self.l_pac, n_seqs = int(first[0]), int(first[1])
            self.anns = []
            for _ in range(n_seqs):
                line = f.readline().rstrip("\n")
                gi, rest = line.split(" ", 1)
                name, _, anno = rest.partition(" ")
                off, ln, na = f.readline().split()
                self.anns.append(Ann(name, anno, int(off), int(ln), int(na)))
        self.crick_l = next((a.offset for a in self.anns if a.is_crick), 0)
        raw = np.fromfile(prefix + ".pac", np.uint8)
        self.pac = raw[: (self.l_pac + 3) // 4].copy()
        # the original (unconverted) bases in the same layout: the methylation calls' reference
        self.opac = (np.fromfile(prefix + ".opac", np.uint8)[: (self.l_pac + 3) // 4].copy()
                     if os.path.exists(prefix + ".opac") else None)

    def pac_codes(self) -> np.ndarray:
        """The forward pac (Watson C->T then Crick G->A) as one code per base."""
        shifts = np.array([6, 4, 2, 0], np.uint8)
        return ((self.pac[:, None] >> shifts) & 3).reshape(-1)[: self.l_pac]
