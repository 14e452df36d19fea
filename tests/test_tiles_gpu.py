"""Extension tile shapes, tile maps and the autotuner on the GPU: any valid map
gives the oracle's tuples, invalid maps are refused, and the autotuner's map
is valid and changes no result."""
import ctypes
import os

import numpy as np
import pytest

import oracle
from bsbolt_gb300 import _lib, autotune, extend, synth

pytestmark = pytest.mark.gpu


def mixed_jobs(seed=5, n_long=300):
    """Queries of every length class up to the 1023-base limit, related and unrelated targets."""
    rng = np.random.Generator(np.random.PCG64(seed))
    parts, rows, base = [], [], 0
    for qlen in list(range(0, 160)) + list(rng.integers(160, 1024, n_long)):
        q = rng.integers(0, 5, qlen).astype(np.uint8)
        if rng.random() < 0.6:
            t = np.concatenate([q, rng.integers(0, 4, int(rng.integers(0, 150))).astype(np.uint8)])
            flip = rng.random(len(t)) < 0.02
            t[flip] = rng.integers(0, 4, int(flip.sum()))
        else:
            t = rng.integers(0, 5, int(rng.integers(0, qlen + 150 + 1))).astype(np.uint8)
        parts += [q, t]
        rows.append((base, base + len(q), len(q), len(t), int(rng.integers(1, 120)),
                     int(rng.choice([0, 3, 50, 100])), int(rng.choice([0, 5, 30])), 0))
        base += len(q) + len(t)
    return np.array(rows, dtype=synth.JOB_DTYPE), np.concatenate(parts)


def random_map(rng, shape_list):
    m = np.zeros(_lib.BSB_TILE_MAP_LEN, np.uint8)
    caps = np.array([g * c for g, c in shape_list])
    for need in range(1, _lib.BSB_TILE_MAP_LEN):
        ok = np.nonzero(caps >= need)[0]
        m[need] = rng.choice(ok)
    return m


def test_random_tile_maps_match_oracle(gpu_ctx):
    jobs, seq = mixed_jobs()
    mat = synth.fill_scmat(1, 4)
    ref, _ = oracle.ksw_batch(jobs, seq, mat, 6, 1, 6, 1, 100, n_threads=os.cpu_count() or 4)
    sl = autotune.shapes()
    rng = np.random.Generator(np.random.PCG64(11))
    try:
        for k in range(4):
            m = random_map(rng, sl)
            autotune.set_map(gpu_ctx, m)
            assert np.array_equal(autotune.get_map(gpu_ctx)[1:], m[1:])
            out = extend.ksw_extend2_batch(gpu_ctx, jobs, seq, mat, 6, 1, 6, 1, 100)
            bad = np.nonzero((out != ref).any(axis=1))[0]
            assert len(bad) == 0, f"map {k}: {len(bad)} tuples differ, first job {bad[:3]}"
    finally:
        autotune.set_map(gpu_ctx, None)
    assert np.array_equal(autotune.get_map(gpu_ctx), autotune.default_map())


def test_tile_map_device_entry_uses_every_mapped_shape(gpu_ctx):
    """The device entry (which cannot see the jobs) runs every shape the map names."""
    torch = pytest.importorskip("torch")
    jobs, seq = mixed_jobs(seed=6, n_long=200)
    mat = synth.fill_scmat(1, 4)
    p = extend.make_param(mat, 6, 1, 6, 1, 100)
    ref, _ = oracle.ksw_batch(jobs, seq, mat, 6, 1, 6, 1, 100, n_threads=8)
    m = random_map(np.random.Generator(np.random.PCG64(12)), autotune.shapes())
    dj = torch.from_numpy(jobs.view(np.uint8).copy()).cuda()
    ds = torch.from_numpy(seq).cuda()
    do = torch.full((len(jobs), 6), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    try:
        autotune.set_map(gpu_ctx, m)
        extend.ksw_extend2_device(gpu_ctx, dj.data_ptr(), len(jobs), ds.data_ptr(), len(seq), p, do.data_ptr())
        _lib.check(gpu_ctx.handle, gpu_ctx.L.bsb_sync(gpu_ctx.handle))
    finally:
        autotune.set_map(gpu_ctx, None)
    assert np.array_equal(do.cpu().numpy(), ref)


def test_invalid_tile_maps_are_refused(gpu_ctx):
    L = gpu_ctx.L
    good = autotune.default_map()
    sl = autotune.shapes()
    small = min(range(len(sl)), key=lambda t: sl[t][0] * sl[t][1])
    bad_cap = good.copy()
    bad_cap[1024] = small                                  # 1024 columns on the smallest shape
    bad_idx = good.copy()
    bad_idx[5] = _lib.BSB_NUM_TILES                        # no such shape
    for m, n in ((bad_cap, len(bad_cap)), (bad_idx, len(bad_idx)), (good, len(good) - 1)):
        rc = L.bsb_set_tile_map(gpu_ctx.handle, m.ctypes.data_as(ctypes.c_void_p), n)
        assert rc == _lib.BSB_EINVAL
        assert np.array_equal(autotune.get_map(gpu_ctx), good)   # the current map stays


def test_autotune_map_is_valid_and_exact(gpu_ctx):
    jobs, seq = synth.ksw_jobs(30000, seed=77)
    mat = synth.fill_scmat(1, 4)
    p = extend.make_param(mat, 6, 1, 6, 1, 100)
    tmap, report = autotune.tune(gpu_ctx, jobs, seq, p, min_jobs=1000, max_jobs=3000, reps=1)
    assert report, "no band had enough jobs"
    sl = autotune.shapes()
    for need in range(1, _lib.BSB_TILE_MAP_LEN):
        g, c = sl[tmap[need]]
        assert g * c >= need
    for r in report:
        assert r["best_ms"] <= r["current_ms"]
    assert np.array_equal(autotune.get_map(gpu_ctx), autotune.default_map())   # tune() restores the map
    ref, _ = oracle.ksw_batch(jobs, seq, mat, 6, 1, 6, 1, 100, n_threads=os.cpu_count() or 4)
    try:
        autotune.set_map(gpu_ctx, tmap)
        out = extend.ksw_extend2_batch(gpu_ctx, jobs, seq, mat, 6, 1, 6, 1, 100)
    finally:
        autotune.set_map(gpu_ctx, None)
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("scoring", [(1, 4, 6, 1, 6, 1, 100), (1, 4, 5, 2, 7, 1, 80), (16, 4, 6, 1, 6, 1, 100)],
                         ids=["bwa_16bit_cells", "asymmetric_gaps_16bit_cells", "a16_32bit_cells"])
def test_every_shape_matches_oracle(gpu_ctx, scoring):
    """Each compiled shape, alone in the map for the query lengths it holds, on jobs of those
    lengths: tuples equal the oracle's.  With a = 16 the scores leave the 16-bit cells' range
    and every shape runs its 32-bit kernel."""
    a, b, o_del, e_del, o_ins, e_ins, zd = scoring
    jobs, seq = mixed_jobs(seed=9, n_long=120)
    mat = synth.fill_scmat(a, b)
    ref, _ = oracle.ksw_batch(jobs, seq, mat, o_del, e_del, o_ins, e_ins, zd, n_threads=os.cpu_count() or 4)
    sl = autotune.shapes()
    base = autotune.default_map()
    need = jobs["qlen"].astype(np.int64) + 1
    try:
        for t, (g, c) in enumerate(sl):
            m = base.copy()
            m[1:g * c + 1] = t
            autotune.set_map(gpu_ctx, m)
            sel = np.nonzero(need <= g * c)[0]
            out = extend.ksw_extend2_batch(gpu_ctx, jobs[sel], seq, mat, o_del, e_del, o_ins, e_ins, zd)
            bad = np.nonzero((out != ref[sel]).any(axis=1))[0]
            assert len(bad) == 0, f"shape {g}x{c}: {len(bad)} tuples differ, first job {sel[bad[:3]]}"
    finally:
        autotune.set_map(gpu_ctx, None)
