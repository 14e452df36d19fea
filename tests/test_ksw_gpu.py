"""Batched ksw_extend2 on the GPU against the reference (golden fixtures) and the
oracle (seeded random jobs), through the C ABI.  Integer DP: bit-exact."""
import glob
import os

import numpy as np
import pytest

import oracle
from bsbolt_gb300 import _lib, extend, synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KSW_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "ksw_*.npz")))

pytestmark = pytest.mark.gpu


def load_ksw(fn):
    d = np.load(fn)
    jobs = np.ascontiguousarray(d["jobs"]).view(synth.JOB_DTYPE).reshape(-1)
    return jobs, d["seq"], d["mat"], [int(x) for x in d["params"]], d["out"]


def assert_same(out, ref, what):
    bad = np.nonzero((out != ref).any(axis=1))[0]
    assert len(bad) == 0, f"{what}: {len(bad)} of {len(ref)} tuples differ; first {bad[:5]}: " \
                          f"gpu {out[bad[:3]].tolist()} ref {ref[bad[:3]].tolist()}"


@pytest.mark.parametrize("fn", KSW_FIXTURES, ids=lambda f: os.path.basename(f))
def test_ksw_golden(gpu_ctx, fn):
    jobs, seq, mat, params, ref = load_ksw(fn)
    out, cells = extend.ksw_extend2_batch(gpu_ctx, jobs, seq, mat, *params, want_cells=True)
    assert_same(out, ref, os.path.basename(fn))
    _, ocells = oracle.ksw_batch(jobs, seq, mat, *params, n_threads=8)
    assert np.array_equal(cells, ocells), "cell counts differ from the reference loop"


@pytest.mark.parametrize("seed", [1, 2])
def test_ksw_random_vs_oracle(gpu_ctx, seed):
    jobs, seq = synth.ksw_jobs(60000, seed=1000 + seed)
    mat = synth.fill_scmat(1, 4)
    out = extend.ksw_extend2_batch(gpu_ctx, jobs, seq, mat, 6, 1, 6, 1, 100)
    ref, _ = oracle.ksw_batch(jobs, seq, mat, 6, 1, 6, 1, 100, n_threads=os.cpu_count() or 4)
    assert_same(out, ref, f"seed {seed}")


def test_ksw_long_queries_all_tiles(gpu_ctx):
    """qlen across every tile width up to the 1023 limit, with bsbolt's end bonus 30."""
    rng = np.random.Generator(np.random.PCG64(3))
    parts, rows, base = [], [], 0
    for qlen in list(range(0, 64)) + list(rng.integers(64, 1024, 400)):
        q = rng.integers(0, 5, qlen).astype(np.uint8)
        if rng.random() < 0.5:
            t = np.concatenate([q, rng.integers(0, 4, int(rng.integers(0, 200))).astype(np.uint8)])
            flip = rng.random(len(t)) < 0.02
            t[flip] = rng.integers(0, 4, int(flip.sum()))
        else:
            t = rng.integers(0, 5, int(rng.integers(0, qlen + 200 + 1))).astype(np.uint8)
        parts += [q, t]
        rows.append((base, base + len(q), len(q), len(t), int(rng.integers(1, 200)),
                     int(rng.choice([0, 1, 5, 50, 100, 200])), 30, 0))
        base += len(q) + len(t)
    jobs = np.array(rows, dtype=synth.JOB_DTYPE)
    seq = np.concatenate(parts)
    mat = synth.fill_scmat(1, 4)
    out = extend.ksw_extend2_batch(gpu_ctx, jobs, seq, mat, 6, 1, 6, 1, 100)
    ref, _ = oracle.ksw_batch(jobs, seq, mat, 6, 1, 6, 1, 100, n_threads=8)
    assert_same(out, ref, "long queries")


@pytest.mark.parametrize("scoring", [(1, 4, 6, 1, 6, 1), (2, 5, 5, 3, 7, 2), (1, 4, 400, 300, 450, 600),
                                     (20, 30, 6, 1, 6, 1)],
                         ids=["bwa", "asym", "wide-penalties", "large-scores"])
def test_ksw_16bit_cell_boundary(gpu_ctx, scoring):
    """Jobs on both sides of the 16-bit cell limit (h0 + qlen * max score around 2047) in
    one batch: the ones below run on 16-bit cells, the ones above on the 32-bit kernel of
    the same shape; penalties or scores too large for the 16-bit arithmetic send the whole
    batch to 32 bits.  Every tuple and cell count must equal the reference loop's."""
    a, b, o_del, e_del, o_ins, e_ins = scoring
    rng = np.random.Generator(np.random.PCG64(17))
    parts, rows, base = [], [], 0
    for k in range(3000):
        qlen = int(rng.integers(1, 300))
        q = rng.integers(0, 4, qlen).astype(np.uint8)
        t = np.concatenate([q, rng.integers(0, 4, int(rng.integers(0, 120))).astype(np.uint8)])
        flip = rng.random(len(t)) < 0.03
        t[flip] = rng.integers(0, 5, int(flip.sum()))
        limit = max(2047 - qlen * a, 10)
        h0 = int(rng.choice([rng.integers(1, 200), limit + int(rng.integers(-3, 4)),
                             int(rng.integers(limit - 2000, limit + 2000))]))
        parts += [q, t]
        rows.append((base, base + qlen, qlen, len(t), max(h0, 1), int(rng.choice([5, 50, 100])), 5, 0))
        base += qlen + len(t)
    jobs = np.array(rows, dtype=synth.JOB_DTYPE)
    seq = np.concatenate(parts)
    mat = synth.fill_scmat(a, b)
    out, cells = extend.ksw_extend2_batch(gpu_ctx, jobs, seq, mat, o_del, e_del, o_ins, e_ins, 100, want_cells=True)
    ref, rcells = oracle.ksw_batch(jobs, seq, mat, o_del, e_del, o_ins, e_ins, 100, n_threads=8)
    assert_same(out, ref, f"16-bit boundary, scoring {scoring}")
    assert np.array_equal(cells, rcells)
    assert (jobs["h0"] + jobs["qlen"] * a > 2047).sum() > 300        # both sides are exercised


def test_ksw_order_invariance_device(gpu_ctx):
    """The issue order (plain bound vs an adversarial cost key) never changes a result."""
    torch = pytest.importorskip("torch")
    jobs, seq = synth.ksw_jobs(20000, seed=99)
    mat = synth.fill_scmat(1, 4)
    p = extend.make_param(mat, 6, 1, 6, 1, 100)
    dj = torch.from_numpy(jobs.view(np.uint8).copy()).cuda()
    ds = torch.from_numpy(seq).cuda()
    outs = []
    torch.cuda.synchronize()   # inputs copied on torch's stream before the context stream reads them
    for cost in (None, torch.arange(len(jobs), dtype=torch.int32, device="cuda"),
                 torch.randint(0, 1 << 30, (len(jobs),), dtype=torch.int32, device="cuda")):
        do = torch.zeros((len(jobs), 6), dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        extend.ksw_extend2_device(gpu_ctx, dj.data_ptr(), len(jobs), ds.data_ptr(), len(seq), p,
                                  do.data_ptr(), 0, cost.data_ptr() if cost is not None else 0)
        torch.cuda.synchronize()
        outs.append(do.cpu().numpy())
    ref, _ = oracle.ksw_batch(jobs, seq, mat, 6, 1, 6, 1, 100, n_threads=8)
    for o in outs:
        assert_same(o, ref, "device entry")


def test_ksw_errors(gpu_ctx):
    jobs, seq = synth.ksw_jobs(10, seed=4)
    mat = synth.fill_scmat(1, 4)
    bad = jobs.copy()
    bad["h0"][3] = 0
    with pytest.raises(_lib.BsbError) as e:
        extend.ksw_extend2_batch(gpu_ctx, bad, seq, mat, 6, 1, 6, 1, 100)
    assert e.value.code == _lib.BSB_EINVAL
    bad = jobs.copy()
    bad["toff"][2] = len(seq)
    with pytest.raises(_lib.BsbError) as e:
        extend.ksw_extend2_batch(gpu_ctx, bad, seq, mat, 6, 1, 6, 1, 100)
    assert e.value.code == _lib.BSB_EINVAL
    with pytest.raises(_lib.BsbError) as e:
        extend.ksw_extend2_batch(gpu_ctx, jobs, seq, mat, 6, 0, 6, 1, 100)
    assert e.value.code == _lib.BSB_EINVAL
    long_q = np.zeros(2000, np.uint8)
    lj = np.array([(0, 0, 2000, 100, 10, 100, 5, 0)], dtype=synth.JOB_DTYPE)
    with pytest.raises(_lib.BsbError) as e:
        extend.ksw_extend2_batch(gpu_ctx, lj, long_q, mat, 6, 1, 6, 1, 100)
    assert e.value.code == _lib.BSB_ETOOLONG
    # the context stays usable after rejected calls
    out = extend.ksw_extend2_batch(gpu_ctx, jobs, seq, mat, 6, 1, 6, 1, 100)
    ref, _ = oracle.ksw_batch(jobs, seq, mat, 6, 1, 6, 1, 100)
    assert_same(out, ref, "after errors")


@pytest.mark.parametrize("reverse", [False, True], ids=["buffer-order", "reversed"])
def test_ksw_host_batch_in_pieces(gpu_ctx, reverse):
    """A host batch of >= 2^20 jobs is extended in pieces whose copies overlap the
    extension; tuples and cell counts still equal the oracle's, whatever the layout."""
    jobs, seq = synth.ksw_jobs((1 << 20) + 12345, seed=4242)
    if reverse:
        jobs = jobs[::-1].copy()
    mat = synth.fill_scmat(1, 4)
    out, cells = extend.ksw_extend2_batch(gpu_ctx, jobs, seq, mat, 6, 1, 6, 1, 100, want_cells=True)
    ref, rcells = oracle.ksw_batch(jobs, seq, mat, 6, 1, 6, 1, 100, n_threads=os.cpu_count() or 4)
    assert_same(out, ref, "pieces")
    assert np.array_equal(cells, rcells)
    assert gpu_ctx.last_kernel_ms() > 0
