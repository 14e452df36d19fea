"""Batched ksw_extend2 on the GPU (host mirror of the reference interface).

``ksw_extend2_batch`` is the batch form of the reference's
``ksw_extend2(qlen, query, tlen, target, m=5, mat, o_del, e_del, o_ins,
e_ins, w, end_bonus, zdrop, h0, &qle, &tle, &gtle, &gscore, &max_off)``
(bsbolt/External/BWA/ksw.c:380-479): same arguments per job, same six
results per job, computed by the sm_103a kernel behind bsb_extend_batch.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .synth import JOB_DTYPE


class Context:
    """One bsb_ctx: a CUDA device, its stream, and device scratch."""

    def __init__(self, device: int = 0):
        self.L = _lib.load()
        self._h = ctypes.c_void_p()
        rc = self.L.bsb_ctx_create(device, ctypes.byref(self._h))
        if rc != 0:
            raise _lib.BsbError(rc, self.L.bsb_strerror(rc).decode())

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return int(self.L.bsb_ctx_stream(self._h) or 0)

    def close(self):
        if self._h:
            self.L.bsb_ctx_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_kernel_ms(self) -> float:
        return float(self.L.bsb_last_kernel_ms(self._h))


def make_param(mat, o_del: int, e_del: int, o_ins: int, e_ins: int, zdrop: int) -> _lib.ExtParam:
    p = _lib.ExtParam()
    m = np.asarray(mat, dtype=np.int8).reshape(25)
    for i in range(25):
        p.mat[i] = int(m[i])
    p.o_del, p.e_del, p.o_ins, p.e_ins, p.zdrop = o_del, e_del, o_ins, e_ins, zdrop
    return p


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def ksw_extend2_batch(ctx: Context, jobs: np.ndarray, seq: np.ndarray, mat, o_del: int,
                      e_del: int, o_ins: int, e_ins: int, zdrop: int, want_cells: bool = False):
    """Run every job of a JOB_DTYPE table through bsb_extend_batch (host buffers).

    Returns out[n, 6] int32 = (score, qle, tle, gtle, gscore, max_off) and,
    with want_cells, the per-job DP cell counts of the reference loop."""
    jobs = np.ascontiguousarray(jobs)
    if jobs.dtype != JOB_DTYPE:
        jobs = jobs.view(JOB_DTYPE).reshape(-1)
    seq = np.ascontiguousarray(seq, dtype=np.uint8)
    n = len(jobs)
    out = np.zeros((n, 6), np.int32)
    cells = np.zeros(n, np.int64) if want_cells else None
    p = make_param(mat, o_del, e_del, o_ins, e_ins, zdrop)
    rc = ctx.L.bsb_extend_batch(ctx.handle, ctypes.byref(p), _ptr(jobs), n, _ptr(seq), len(seq),
                                _ptr(out), _ptr(cells) if want_cells else None)
    _lib.check(ctx.handle, rc)
    return (out, cells) if want_cells else out


def ksw_extend2_device(ctx: Context, d_jobs: int, n: int, d_seq: int, seq_bytes: int, param,
                       d_out: int, d_cells: int = 0, d_cost: int = 0):
    """Device-buffer form (raw device pointers, e.g. torch ``data_ptr()``); asynchronous
    on the context stream."""
    rc = ctx.L.bsb_extend_batch_device(ctx.handle, ctypes.byref(param), ctypes.c_void_p(d_jobs), n,
                                       ctypes.c_void_p(d_seq), seq_bytes,
                                       ctypes.c_void_p(d_cost) if d_cost else None,
                                       ctypes.c_void_p(d_out), ctypes.c_void_p(d_cells) if d_cells else None)
    _lib.check(ctx.handle, rc)
