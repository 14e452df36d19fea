"""Mate-rescue Smith-Waterman on the GPU (host mirror of ksw_align2).

``align2_batch`` is ksw_align2 (bsbolt/External/BWA/ksw.c:336-360) for many jobs at
once, as mem_matesw calls it (bwamem_pair.c:150-151); it goes through the C ABI
(bsb_align2_batch) of libbsbgpu.so.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .extend import Context, _ptr, make_param

JOB_DTYPE = np.dtype([("qoff", "<i8"), ("toff", "<i8"), ("qlen", "<i4"), ("tlen", "<i4"), ("xtra", "<i4"),
                      ("pad", "<i4")])                                     # bsb_sw_job_t
KSWR_DTYPE = np.dtype([("score", "<i4"), ("te", "<i4"), ("qe", "<i4"), ("score2", "<i4"), ("te2", "<i4"),
                       ("tb", "<i4"), ("qb", "<i4")])                      # bsb_kswr_t (kswr_t)
KSW_XBYTE, KSW_XSTOP, KSW_XSUBO, KSW_XSTART = 0x10000, 0x20000, 0x40000, 0x80000
MAX_QLEN = 1024


def matesw_xtra(qlen: int, a: int = 1, min_seed_len: int = 19) -> int:
    """The flags mem_matesw passes (bwamem_pair.c:149)."""
    return KSW_XSUBO | KSW_XSTART | (KSW_XBYTE if qlen * a < 250 else 0) | (min_seed_len * a)


def align2_batch(ctx: Context, jobs: np.ndarray, seq: np.ndarray, mat, o_del: int, e_del: int, o_ins: int,
                 e_ins: int) -> np.ndarray:
    """ksw_align2 for every job (JOB_DTYPE); returns kswr_t records (KSWR_DTYPE)."""
    jobs = np.ascontiguousarray(jobs, dtype=JOB_DTYPE)
    seq = np.ascontiguousarray(seq, dtype=np.uint8)
    out = np.empty(len(jobs), KSWR_DTYPE)
    p = make_param(mat, o_del, e_del, o_ins, e_ins, 0)
    import ctypes
    rc = ctx.L.bsb_align2_batch(ctx.handle, ctypes.byref(p), _ptr(jobs) if len(jobs) else None, len(jobs),
                                _ptr(seq) if len(seq) else None, len(seq), _ptr(out) if len(jobs) else None)
    _lib.check(ctx.handle, rc)
    return out


def _main(argv=None) -> None:
    """Times align2_batch on seeded mem_matesw-shaped jobs (synth.matesw_jobs): one line
    per repetition with the wall time of the call (copies included) and its forward-pass
    cells per second (padded query columns x target rows, as the striped code computes)."""
    import argparse
    import time

    from . import synth
    ap = argparse.ArgumentParser(prog="python -m bsbolt_gb300.matesw")
    ap.add_argument("--jobs", type=int, default=40000)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)
    jobs, seq = synth.matesw_jobs(args.jobs)
    mat = synth.fill_scmat(1, 4)
    ctx = Context(args.device)
    p = np.where(jobs["xtra"] & KSW_XBYTE, 16, 8)
    cells = float(((jobs["qlen"] + p - 1) // p * p).astype(np.float64) @ jobs["tlen"].astype(np.float64))
    for r in range(args.reps):
        t0 = time.perf_counter()
        align2_batch(ctx, jobs, seq, mat, 6, 1, 6, 1)
        dt = time.perf_counter() - t0
        print(f"rep {r}: {args.jobs} jobs {dt * 1e3:.3f} ms {args.jobs / dt:.0f} jobs/s {cells / dt / 1e9:.2f} GCUPS")


if __name__ == "__main__":
    _main()
