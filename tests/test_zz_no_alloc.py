"""The allocation-free extension entry point (bsb_extend_batch_noalloc).

For callers that may not call cudaMalloc (a host application's memory
manager owns the device, or cudaMalloc's implicit synchronisation is not
allowed where they run): the entry point keeps its scheduling scratch in one
fixed device array of the library.  This test calls it through the C ABI
twice in a row, on buffers the test allocates, and checks both results
against the context-based entry point bsb_extend_batch (integer DP: the
tolerance is zero).  It is collected last on purpose and must pass alone in
a fresh process as well as after the other tests.
"""
import ctypes

import numpy as np
import pytest

from bsbolt_gb300 import _lib, extend, synth

pytestmark = pytest.mark.gpu


def _run_noalloc(L, jobs, seq, param, stream):
    import torch
    dj = torch.from_numpy(jobs.view(np.uint8).reshape(-1).copy()).cuda()
    ds = torch.from_numpy(seq).cuda()
    do = torch.full((len(jobs), 6), -7, dtype=torch.int32, device="cuda")
    dc = torch.zeros(len(jobs), dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    rc = L.bsb_extend_batch_noalloc(ctypes.byref(param), ctypes.c_void_p(dj.data_ptr()), len(jobs),
                                    ctypes.c_void_p(ds.data_ptr()), len(seq), ctypes.c_void_p(do.data_ptr()),
                                    ctypes.c_void_p(dc.data_ptr()), ctypes.c_void_p(stream))
    assert rc == 0, _lib.load().bsb_strerror(rc)
    torch.cuda.synchronize()
    return do.cpu().numpy(), dc.cpu().numpy()


def test_noalloc_matches_context_entry_twice():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    mat = synth.fill_scmat(1, 4)
    param = extend.make_param(mat, 6, 1, 6, 1, 100)
    ctx = extend.Context(0)
    try:
        stream = torch.cuda.current_stream().cuda_stream
        for seed in (31, 32):          # two calls in a row reuse the same fixed scratch
            jobs, seq = synth.ksw_jobs(20000 + 1000 * seed, seed=seed)
            out, cells = _run_noalloc(L, jobs, seq, param, stream)
            ref, rcells = extend.ksw_extend2_batch(ctx, jobs, seq, mat, 6, 1, 6, 1, 100, want_cells=True)
            assert np.array_equal(out, ref), f"call with seed {seed}: tuples differ from bsb_extend_batch"
            assert np.array_equal(cells, rcells)
    finally:
        ctx.close()


def test_noalloc_rejects_oversized_batch():
    L = _lib.load()
    param = extend.make_param(synth.fill_scmat(1, 4), 6, 1, 6, 1, 100)
    rc = L.bsb_extend_batch_noalloc(ctypes.byref(param), ctypes.c_void_p(16), _lib.BSB_NOALLOC_MAX_JOBS + 1,
                                    ctypes.c_void_p(16), 1, ctypes.c_void_p(16), None, None)
    assert rc == _lib.BSB_ECAPACITY
