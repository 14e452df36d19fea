"""Tile-shape autotuner of the batched extension (no counterpart in the reference).

A batched ``ksw_extend2`` job runs on a tile of G lanes x C query columns per
lane (32/G jobs per warp); the library compiles ``BSB_NUM_TILES`` shapes and a
tile map assigns one to every query length (``include/bsbgpu.h``).  This
module measures, on the caller's own jobs and GPU, every compiled shape that
holds a band of query lengths, through the library's own extension entry point
(``bsb_extend_batch``, device time from ``bsb_last_kernel_ms``), and keeps the
fastest per band.  A shape never changes a result; each candidate's tuples are
still compared with the current map's before it may win.

    ctx = extend.Context(0)
    tmap, report = autotune.tune(ctx, jobs, seq, param)
    autotune.set_map(ctx, tmap)            # or save_map(path, ...) / load_map(path)
"""
from __future__ import annotations

import ctypes
import json

import numpy as np

from . import _lib
from .synth import JOB_DTYPE


def shapes(L=None) -> list[tuple[int, int]]:
    """The compiled tile shapes (G, C), indexed by shape number."""
    L = L or _lib.load()
    G = (ctypes.c_int32 * _lib.BSB_NUM_TILES)()
    C = (ctypes.c_int32 * _lib.BSB_NUM_TILES)()
    n = L.bsb_tile_shapes(G, C, _lib.BSB_NUM_TILES)
    return [(G[t], C[t]) for t in range(n)]


def default_map(L=None) -> np.ndarray:
    L = L or _lib.load()
    m = np.zeros(_lib.BSB_TILE_MAP_LEN, np.uint8)
    rc = L.bsb_get_tile_map(None, m.ctypes.data_as(ctypes.c_void_p), len(m))
    if rc:
        raise _lib.BsbError(rc, "bsb_get_tile_map")
    return m


def get_map(ctx) -> np.ndarray:
    m = np.zeros(_lib.BSB_TILE_MAP_LEN, np.uint8)
    _lib.check(ctx.handle, ctx.L.bsb_get_tile_map(ctx.handle, m.ctypes.data_as(ctypes.c_void_p), len(m)))
    return m


def set_map(ctx, tmap) -> None:
    """Install a tile map on ctx (None restores the built-in default)."""
    if tmap is None:
        _lib.check(ctx.handle, ctx.L.bsb_set_tile_map(ctx.handle, None, 0))
        return
    m = np.ascontiguousarray(tmap, dtype=np.uint8)
    _lib.check(ctx.handle, ctx.L.bsb_set_tile_map(ctx.handle, m.ctypes.data_as(ctypes.c_void_p), len(m)))


def bands(max_need: int = _lib.BSB_TILE_MAP_LEN - 1) -> list[tuple[int, int]]:
    """Query-length bands tuned as one unit, as inclusive need = qlen + 1 ranges:
    8 columns wide up to 64, 16 up to 256, 64 beyond."""
    out, lo = [], 1
    while lo <= max_need:
        width = 8 if lo <= 64 else (16 if lo <= 256 else 64)
        hi = min(lo + width - 1, max_need)
        out.append((lo, hi))
        lo = hi + 1
    return out


def candidates(shape_list, lo: int, hi: int, slack: float = 1.6) -> list[int]:
    """Shapes that hold the band's widest query without more than `slack` x its columns."""
    cap = max(hi, int(hi * slack))
    return [t for t, (g, c) in enumerate(shape_list) if hi <= g * c <= max(cap, hi + 8)]


def _compact(jobs: np.ndarray, seq: np.ndarray):
    """The jobs with their query/target bytes copied into a buffer of their own."""
    q = [seq[j["qoff"]:j["qoff"] + j["qlen"]] for j in jobs]
    t = [seq[j["toff"]:j["toff"] + j["tlen"]] for j in jobs]
    ql = jobs["qlen"].astype(np.int64)
    tl = jobs["tlen"].astype(np.int64)
    qoff = np.concatenate([[0], np.cumsum(ql)[:-1]]) if len(jobs) else ql
    toff = ql.sum() + (np.concatenate([[0], np.cumsum(tl)[:-1]]) if len(jobs) else tl)
    buf = np.concatenate(q + t) if len(jobs) else np.zeros(0, np.uint8)
    out = jobs.copy()
    out["qoff"], out["toff"] = qoff, toff
    return out, np.ascontiguousarray(buf, dtype=np.uint8)


def _run(ctx, param, jobs, seq):
    n = len(jobs)
    out = np.zeros((n, 6), np.int32)
    rc = ctx.L.bsb_extend_batch(ctx.handle, ctypes.byref(param), jobs.ctypes.data_as(ctypes.c_void_p), n,
                                seq.ctypes.data_as(ctypes.c_void_p), len(seq), out.ctypes.data_as(ctypes.c_void_p),
                                None)
    _lib.check(ctx.handle, rc)
    return out, float(ctx.L.bsb_last_kernel_ms(ctx.handle))


def tune(ctx, jobs: np.ndarray, seq: np.ndarray, param, min_jobs: int = 4096, max_jobs: int = 200_000,
         reps: int = 3, slack: float = 1.6, seed: int = 1):
    """Measure the candidate shapes of every band with at least `min_jobs` jobs.

    Returns (tile map, report); bands with too few jobs keep the context's
    current shape.  The context's map is left as it was."""
    jobs = np.ascontiguousarray(jobs)
    if jobs.dtype != JOB_DTYPE:
        jobs = jobs.view(JOB_DTYPE).reshape(-1)
    seq = np.ascontiguousarray(seq, dtype=np.uint8)
    shape_list = shapes(ctx.L)
    base = get_map(ctx)
    tmap = base.copy()
    need = jobs["qlen"].astype(np.int64) + 1
    rng = np.random.Generator(np.random.PCG64(seed))
    report = []
    try:
        for lo, hi in bands():
            idx = np.nonzero((need >= lo) & (need <= hi))[0]
            if len(idx) < min_jobs:
                continue
            if len(idx) > max_jobs:
                idx = np.sort(rng.choice(idx, max_jobs, replace=False))
            bj, bs = _compact(jobs[idx], seq)
            cands = candidates(shape_list, lo, hi, slack)
            cur = int(base[hi])
            if cur not in cands:
                cands.append(cur)
            ref_out, times = None, {}
            for t in [cur] + [c for c in cands if c != cur]:
                trial = base.copy()
                trial[lo:hi + 1] = t
                set_map(ctx, trial)
                ms = []
                for r in range(reps + 1):
                    out, k = _run(ctx, param, bj, bs)
                    if r:
                        ms.append(k)
                if ref_out is None:
                    ref_out = out
                elif not np.array_equal(out, ref_out):
                    raise AssertionError(f"tile shape {shape_list[t]} changed results for need {lo}-{hi}")
                times[t] = float(np.median(ms))
            best = min(times, key=times.get)
            tmap[lo:hi + 1] = best
            report.append({"need": [lo, hi], "jobs": int(len(idx)), "current": list(shape_list[cur]),
                           "best": list(shape_list[best]), "current_ms": round(times[cur], 4),
                           "best_ms": round(times[best], 4),
                           "ms": {f"{shape_list[t][0]}x{shape_list[t][1]}": round(v, 4) for t, v in times.items()}})
    finally:
        set_map(ctx, base)
    return tmap, report


def save_map(path: str, tmap, report=None) -> None:
    sl = shapes()
    json.dump({"tile_map": [int(x) for x in tmap], "shapes": [list(s) for s in sl], "report": report or []},
              open(path, "w"))


def load_map(path: str) -> np.ndarray:
    d = json.load(open(path))
    if [list(s) for s in shapes()] != d["shapes"]:
        raise ValueError(f"{path} was tuned for another set of tile shapes")
    return np.asarray(d["tile_map"], dtype=np.uint8)
