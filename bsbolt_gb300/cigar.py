"""CIGAR, MD and methylation strings on the GPU (host mirror of bwa_gen_cigar2).

``gen_cigar_batch`` is bwa_gen_cigar2 (bsbolt/External/BWA/bwa.c:199-351) for many
alignments at once, each called as mem_reg2aln calls it (bwamem.c:1228); it goes
through the C ABI (bsb_gen_cigar_batch) of libbsbgpu.so.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .extend import Context

JOB_DTYPE = np.dtype([("rb", "<i8"), ("re", "<i8"), ("qoff", "<i8"), ("ooff", "<i8"),
                      ("l_query", "<i4"), ("w", "<i4")])                  # bsb_cigar_job_t
OUT_DTYPE = np.dtype([("score", "<i4"), ("n_cigar", "<i4"), ("NM", "<i4"), ("cg_meth", "<i4"),
                      ("cg_unmeth", "<i4"), ("ch_meth", "<i4"), ("ch_unmeth", "<i4"), ("status", "<i4"),
                      ("off", "<i8"), ("bytes", "<i4"), ("pad", "<i4")])   # bsb_cigar_out_t
OK, REJECT, NO_MD, CLIPPED, BAND_EXIT = 0, 1, 2, 3, 4
MAX_LEN = 1024


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def upload_opac(ctx: Context, opac: np.ndarray, l_pac: int) -> None:
    """bsb_index_upload_opac: the original (unconverted) 2-bit reference of a loaded index."""
    opac = np.ascontiguousarray(opac, dtype=np.uint8)
    _lib.check(ctx.handle, ctx.L.bsb_index_upload_opac(ctx.handle, _ptr(opac), int(l_pac)))


def gen_cigar_batch(ctx: Context, jobs: np.ndarray, qbuf: np.ndarray, obuf: np.ndarray, crick_l: int,
                    opt: "_lib.AlignOpt" = None):
    """bwa_gen_cigar2 for every job (JOB_DTYPE).  Returns (out[OUT_DTYPE], blob uint8):
    for status OK a job's bytes blob[off:off+bytes] are its CIGAR words (uint32,
    len<<4|op) followed by the NUL-terminated "MD\\tXB:Z:calls" string; NO_MD has the
    words only; the other statuses have no bytes."""
    jobs = np.ascontiguousarray(jobs, dtype=JOB_DTYPE)
    qbuf = np.ascontiguousarray(qbuf, dtype=np.uint8)
    obuf = np.ascontiguousarray(obuf, dtype=np.uint8)
    opt = opt or _lib.AlignOpt.bwa_defaults()
    n = len(jobs)
    out = np.empty(n, OUT_DTYPE)
    # the device's per-job output bound (14 bytes per base of either sequence + 48); rejected
    # jobs write nothing, so clipping their lengths only loosens the bound
    cap = 14 * (int(np.clip(jobs["l_query"], 0, MAX_LEN).sum(dtype=np.int64)) +
                int(np.clip(jobs["re"] - jobs["rb"], 0, MAX_LEN).sum(dtype=np.int64))) + 48 * n + 64
    blob = getattr(ctx, "_cigar_blob", None)
    if blob is None or len(blob) < cap:
        blob = np.empty(cap, np.uint8)
        ctx._cigar_blob = blob
    used = ctypes.c_int64(0)
    rc = ctx.L.bsb_gen_cigar_batch(ctx.handle, ctypes.byref(opt), int(crick_l), n,
                                   _ptr(jobs) if n else None, _ptr(qbuf) if len(qbuf) else None, len(qbuf),
                                   _ptr(obuf) if len(obuf) else None, len(obuf), _ptr(out) if n else None,
                                   _ptr(blob), cap, ctypes.byref(used))
    _lib.check(ctx.handle, rc)
    return out, blob[: used.value].copy()


def record(out_i, blob: np.ndarray):
    """(CIGAR words uint32[n_cigar], text bytes without the NUL) of one job's record."""
    b = bytes(blob[out_i["off"]: out_i["off"] + out_i["bytes"]])
    k = 4 * int(out_i["n_cigar"]) if out_i["status"] in (OK, NO_MD) else 0
    words = np.frombuffer(b[:k], np.uint32)
    return words, b[k:].rstrip(b"\0")
