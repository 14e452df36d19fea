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


def last_extensions(ctx: Context) -> int:
    """bwt_extend calls (one bwt_2occ4 each) of the context's most recent seeding batch."""
    v = ctypes.c_int64()
    _lib.check(ctx.handle, ctx.L.bsb_last_seed_extensions(ctx.handle, ctypes.byref(v)))
    return int(v.value)


def set_read_order_keys(ctx: Context, keys) -> None:
    """Orders the next alignment batch (of len(keys) reads) by these per-read keys, larger
    first (bsb_set_read_order_keys); None clears."""
    if keys is None:
        _lib.check(ctx.handle, ctx.L.bsb_set_read_order_keys(ctx.handle, None, 0))
        return
    k = np.ascontiguousarray(np.minimum(np.asarray(keys, np.int64), 2**31 - 1), dtype=np.int32)
    _lib.check(ctx.handle, ctx.L.bsb_set_read_order_keys(ctx.handle, _ptr(k), len(k)))


ALIGN_STAGES = ("seeding", "sa_rows", "chains", "chain2aln", "dedup", "d2h")


def last_stage_ms(ctx: Context) -> dict:
    """Device ms per stage of the context's last alignment batch (bsb_last_stage_ms)."""
    ms = np.zeros(_lib.BSB_ALIGN_STAGES, np.float32)
    _lib.check(ctx.handle, ctx.L.bsb_last_stage_ms(ctx.handle, _ptr(ms), len(ms)))
    return dict(zip(ALIGN_STAGES, (float(x) for x in ms)))


def sa_batch(ctx: Context, rows: np.ndarray) -> np.ndarray:
    rows = np.ascontiguousarray(rows, dtype=np.uint64)
    pos = np.zeros(len(rows), np.uint64)
    _lib.check(ctx.handle, ctx.L.bsb_sa_batch(ctx.handle, _ptr(rows), len(rows), _ptr(pos)))
    return pos


# bsb_reg_t: the mem_alnreg_t fields mem_chain2aln sets (bwamem.h:64-82)
REG_DTYPE = np.dtype([("rb", "<i8"), ("re", "<i8"), ("qb", "<i4"), ("qe", "<i4"), ("rid", "<i4"),
                      ("score", "<i4"), ("truesc", "<i4"), ("w", "<i4"), ("seedcov", "<i4"),
                      ("seedlen0", "<i4"), ("frac_rep", "<f4"), ("n_comp", "<i4")])


def align_regs(ctx: Context, seqs: np.ndarray, offs: np.ndarray, opt: "_lib.AlignOpt" = None, dedup: bool = False):
    """Seeds -> chains -> chain filter -> mem_chain2aln for every read (the pre-dedup part of
    mem_align1_core, bwamem.c:1157-1180) on the GPU; with dedup, mem_sort_dedup_patch too
    (bsb_mem_align1_batch: the regions mem_align1_core returns, bwamem.c:1157-1188).
    Returns (regs[REG_DTYPE], regs_off[n+1])."""
    seqs = np.ascontiguousarray(seqs, dtype=np.uint8)
    offs = np.ascontiguousarray(offs, dtype=np.int64)
    opt = opt or _lib.AlignOpt.bwa_defaults()
    n = len(offs) - 1
    cap = int(offs[-1] - offs[0]) * 4 + 64 * max(n, 1)
    # the worst-case region buffer is large and mostly unused: keep one per context and
    # hand back a copy of the part the call filled
    regs = getattr(ctx, "_regs_buf", None)
    if regs is None or len(regs) < cap:
        regs = np.empty(cap, REG_DTYPE)
        ctx._regs_buf = regs
    regs_off = np.empty(n + 1, np.int64)
    fn = ctx.L.bsb_mem_align1_batch if dedup else ctx.L.bsb_align_regs_batch
    rc = fn(ctx.handle, ctypes.byref(opt), n, _ptr(seqs) if len(seqs) else None, _ptr(offs), _ptr(regs), cap,
            _ptr(regs_off))
    if rc == _lib.BSB_ECAPACITY and regs_off[-1] > cap:    # more regions than the first guess: size and rerun
        cap = int(regs_off[-1])
        regs = np.empty(cap, REG_DTYPE)
        ctx._regs_buf = regs
        rc = fn(ctx.handle, ctypes.byref(opt), n, _ptr(seqs) if len(seqs) else None, _ptr(offs), _ptr(regs), cap,
                _ptr(regs_off))
    _lib.check(ctx.handle, rc)
    return regs[: regs_off[-1]].copy(), regs_off


def read_cost_log(ctx: Context, enable: bool = True) -> None:
    """bsb_read_cost_log: keep each later alignment batch's per-read features and DP cells."""
    _lib.check(ctx.handle, ctx.L.bsb_read_cost_log(ctx.handle, int(enable)))


def last_read_costs(ctx: Context, n_reads: int):
    """(features[n, 8] float32, cells[n] int64) of the last logged alignment batch."""
    feat = np.zeros((n_reads, 8), np.float32)
    cells = np.zeros(n_reads, np.int64)
    _lib.check(ctx.handle, ctx.L.bsb_last_read_costs(ctx.handle, n_reads, _ptr(feat), _ptr(cells)))
    return feat, cells


def set_read_cost_model(ctx: Context, model=None) -> None:
    """Order the reads of later alignment batches by the cost model's prediction (a
    cost_model.CostModel, whose device weights must stay alive meanwhile); None restores the
    chain-count order."""
    ptr = ctypes.c_void_p(model.w.data_ptr()) if model is not None else None
    _lib.check(ctx.handle, ctx.L.bsb_set_read_cost_model(ctx.handle, ptr))
