"""SMEM seeding and suffix-array lookups on the GPU (host mirror of the reference calls).

``seed_batch`` is mem_collect_intv (bsbolt/External/BWA/bwamem.c:118-166) for
many reads at once; ``sa_batch`` is bwt_sa (bwt.c:86-96) for many rows.
Both go through the C ABI (bsb_seed_batch / bsb_sa_batch) of libbsbgpu.so.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .extend import Context


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def load_index(ctx: Context, prefix: str) -> None:
    """bsb_index_load: read <prefix>.bwt/.sa/.ann/.pac and keep them in device memory."""
    _lib.check(ctx.handle, ctx.L.bsb_index_load(ctx.handle, prefix.encode()))


def seed_batch(ctx: Context, seqs: np.ndarray, offs: np.ndarray, min_seed_len: int = 19,
               split_factor: float = 1.5, split_width: int = 10, max_mem_intv: int = 20):
    """Seeds of every read (nt4 codes, read r = seqs[offs[r]:offs[r+1]]).

    Returns (intervals[m, 4] uint64 = x0, x1, x2, info; out_off[n+1])."""
    seqs = np.ascontiguousarray(seqs, dtype=np.uint8)
    offs = np.ascontiguousarray(offs, dtype=np.int64)
    n = len(offs) - 1
    total = int(offs[-1] - offs[0])
    cap = 2 * total + 32 * max(n, 1)
    out = np.zeros((cap, 4), np.uint64)
    out_off = np.zeros(n + 1, np.int64)
    opt = _lib.SeedOpt(min_seed_len, split_factor, split_width, max_mem_intv)
    rc = ctx.L.bsb_seed_batch(ctx.handle, ctypes.byref(opt), n, _ptr(seqs) if len(seqs) else None,
                              _ptr(offs), _ptr(out), cap, _ptr(out_off))
    _lib.check(ctx.handle, rc)
    return out[: out_off[-1]].copy(), out_off


def sa_batch(ctx: Context, rows: np.ndarray) -> np.ndarray:
    rows = np.ascontiguousarray(rows, dtype=np.uint64)
    pos = np.zeros(len(rows), np.uint64)
    _lib.check(ctx.handle, ctx.L.bsb_sa_batch(ctx.handle, _ptr(rows), len(rows), _ptr(pos)))
    return pos
