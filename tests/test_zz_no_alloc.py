"""The allocation-free extension entry point (bsb_extend_batch_noalloc).

For callers that may not call cudaMalloc (a host application's memory
manager owns the device, or cudaMalloc's implicit synchronisation is not
allowed where they run): the entry point keeps its scheduling scratch in one
fixed device array of the library.  These tests call it through the C ABI
twice in a row, on buffers the test allocates, and check both results
against the CPU oracle and the context-based entry point bsb_extend_batch
(integer DP: the tolerance is zero), with 16-bit and 32-bit cells, with and
without the per-job cell counts, with a job that fails the preconditions
(its slot stays as it was), and that a call leaves the device's free memory
and torch's allocator as they were.  Collected last on purpose; they pass
alone in a fresh process as well as after the other tests.
"""
import ctypes
import os

import numpy as np
import pytest

import oracle
from bsbolt_gb300 import _lib, extend, synth

pytestmark = pytest.mark.gpu

SCORINGS = {"bwa": (1, 4, 6, 1, 6, 1, 100),          # 16-bit cells
            "a16": (16, 4, 6, 1, 6, 1, 100)}         # scores above 15: 32-bit cells


def _buffers(jobs, seq):
    import torch
    dj = torch.from_numpy(jobs.view(np.uint8).reshape(-1).copy()).cuda()
    ds = torch.from_numpy(seq).cuda()
    do = torch.full((len(jobs), 6), -7, dtype=torch.int32, device="cuda")
    dc = torch.zeros(len(jobs), dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    return dj, ds, do, dc


def _call(L, param, dj, n, ds, seq_bytes, do, dc, stream):
    rc = L.bsb_extend_batch_noalloc(ctypes.byref(param), ctypes.c_void_p(dj.data_ptr()), n,
                                    ctypes.c_void_p(ds.data_ptr()), seq_bytes, ctypes.c_void_p(do.data_ptr()),
                                    ctypes.c_void_p(dc.data_ptr()) if dc is not None else None,
                                    ctypes.c_void_p(stream))
    assert rc == 0, L.bsb_strerror(rc)


@pytest.mark.parametrize("name", list(SCORINGS))
def test_noalloc_matches_oracle_and_context_entry_twice(name):
    torch = pytest.importorskip("torch")
    a, b, o_del, e_del, o_ins, e_ins, zd = SCORINGS[name]
    L = _lib.load()
    mat = synth.fill_scmat(a, b)
    param = extend.make_param(mat, o_del, e_del, o_ins, e_ins, zd)
    ctx = extend.Context(0)
    try:
        stream = torch.cuda.current_stream().cuda_stream
        for seed, with_cells in ((31, True), (32, False)):   # two calls in a row share the fixed scratch
            jobs, seq = synth.ksw_jobs(20000 + 1000 * seed, seed=seed)
            dj, ds, do, dc = _buffers(jobs, seq)
            _call(L, param, dj, len(jobs), ds, len(seq), do, dc if with_cells else None, stream)
            torch.cuda.synchronize()
            out, cells = do.cpu().numpy(), dc.cpu().numpy()
            ref, rcells = oracle.ksw_batch(jobs, seq, mat, o_del, e_del, o_ins, e_ins, zd,
                                           n_threads=os.cpu_count() or 4)
            assert np.array_equal(out, ref), f"seed {seed}: tuples differ from the oracle"
            ctx_out, ctx_cells = extend.ksw_extend2_batch(ctx, jobs, seq, mat, o_del, e_del, o_ins, e_ins, zd,
                                                          want_cells=True)
            assert np.array_equal(out, ctx_out), f"seed {seed}: tuples differ from bsb_extend_batch"
            if with_cells:
                assert np.array_equal(cells, rcells) and np.array_equal(cells, ctx_cells)
            else:
                assert not cells.any()                      # d_cells NULL: nothing written there
    finally:
        ctx.close()


def test_noalloc_skips_a_job_that_fails_the_preconditions():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    mat = synth.fill_scmat(1, 4)
    param = extend.make_param(mat, 6, 1, 6, 1, 100)
    jobs, seq = synth.ksw_jobs(3000, seed=41)
    bad = 1234
    jobs["h0"][bad] = 0                                      # the reference asserts h0 > 0
    dj, ds, do, dc = _buffers(jobs, seq)
    _call(L, param, dj, len(jobs), ds, len(seq), do, dc, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    out = do.cpu().numpy()
    assert (out[bad] == -7).all()                            # its slot is left as it was
    keep = np.arange(len(jobs)) != bad
    ref, _ = oracle.ksw_batch(jobs[keep], seq, mat, 6, 1, 6, 1, 100, n_threads=os.cpu_count() or 4)
    assert np.array_equal(out[keep], ref)


def test_noalloc_allocates_nothing():
    """After a warm-up call (the CUDA runtime loads the kernels' code on their first launch),
    a call changes neither the device's free memory nor torch's allocator."""
    torch = pytest.importorskip("torch")
    L = _lib.load()
    param = extend.make_param(synth.fill_scmat(1, 4), 6, 1, 6, 1, 100)
    jobs, seq = synth.ksw_jobs(50000, seed=43)
    dj, ds, do, dc = _buffers(jobs, seq)
    stream = torch.cuda.current_stream().cuda_stream
    _call(L, param, dj, len(jobs), ds, len(seq), do, dc, stream)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0, reserved0 = torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
    for _ in range(3):
        _call(L, param, dj, len(jobs), ds, len(seq), do, dc, stream)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"device free memory moved by {free0 - free1} bytes"
    assert torch.cuda.memory_allocated() == alloc0 and torch.cuda.memory_reserved() == reserved0


def test_noalloc_rejects_oversized_batch():
    L = _lib.load()
    param = extend.make_param(synth.fill_scmat(1, 4), 6, 1, 6, 1, 100)
    rc = L.bsb_extend_batch_noalloc(ctypes.byref(param), ctypes.c_void_p(16), _lib.BSB_NOALLOC_MAX_JOBS + 1,
                                    ctypes.c_void_p(16), 1, ctypes.c_void_p(16), None, None)
    assert rc == _lib.BSB_ECAPACITY
