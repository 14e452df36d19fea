"""The suffixes sorted on the GPU give the reference `bwa index` files byte for byte
(tests/golden/index*_sha256.json, which the reference produced) and the host SA-IS order on
texts with long repeats: bsb_build_suffix_array (prefix doubling, 32-bit ranks, the whole
array) and bsb_build_bwt (64-bit ranks in chunks; the BWT and sampled rows), the latter also
with chunks small enough that every round takes many of them."""
import ctypes
import hashlib
import json
import os
import sys

import numpy as np
import pytest

from bsbolt_gb300 import _lib, index, synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import golden_data  # noqa: E402

pytestmark = pytest.mark.gpu


def sha(fn):
    return hashlib.sha256(open(fn, "rb").read()).hexdigest()


@pytest.mark.parametrize("chunk", [0, 50_000, 400_000], ids=["one-chunk", "chunks-50k", "chunks-400k"])
@pytest.mark.parametrize("gen,fixture", [(golden_data.golden_genome, "index_sha256.json"),
                                         (golden_data.golden_genome_rep, "index_rep_sha256.json")],
                         ids=["plain", "repeats"])
def test_gpu_suffix_array_gives_reference_index_files(gpu_ctx, tmp_path, gen, fixture, chunk):
    fa = str(tmp_path / "ref.fa")
    synth.write_fasta(fa, gen())
    index.build_index(fa, str(tmp_path / "ref"), ctx=gpu_ctx, chunk=chunk)
    want = json.load(open(os.path.join(GOLDEN, fixture)))["files"]
    for ext, h in want.items():
        assert sha(str(tmp_path / "ref") + "." + ext) == h, f".{ext} differs from the reference bwa index"


def test_gpu_suffix_array_matches_sais(gpu_ctx):
    """Random texts, one long run and a period-7 text, so the doubling needs many rounds."""
    rng = np.random.Generator(np.random.PCG64(3))
    for l_pac in (1, 2, 3, 17, 64, 1000, 5000):
        for kind in range(3):
            b = rng.integers(0, 4, l_pac).astype(np.uint8)
            if kind == 1:
                b[:] = b[0]
            elif kind == 2:
                b = np.resize(rng.integers(0, 4, 7), l_pac).astype(np.uint8)
            pac = np.zeros((l_pac + 3) // 4, np.uint8)
            for i, x in enumerate(b):
                pac[i >> 2] |= int(x) << ((~i & 3) << 1)
            sa = np.empty(2 * l_pac + 1, np.int64)
            _lib.check(gpu_ctx.handle, gpu_ctx.L.bsb_build_suffix_array(
                gpu_ctx.handle, pac.ctypes.data_as(ctypes.c_void_p), l_pac, sa.ctypes.data_as(ctypes.c_void_p)))
            text = np.concatenate([b, 3 - b[::-1]]).astype(np.uint8)
            assert np.array_equal(sa, index.suffix_array(text).astype(np.int64)), (l_pac, kind)


def test_gpu_bwt_matches_sais(gpu_ctx):
    """bsb_build_bwt on random texts, one long run, a period-7 text and a text of a repeated unit
    with 1 % changes, against the BWT and sampled rows of the host SA-IS order, with one chunk and
    with chunks of a few hundred suffixes (a text whose 5-symbol buckets do not fit is refused)."""
    rng = np.random.Generator(np.random.PCG64(5))
    for l_pac in (1, 2, 3, 17, 64, 1000, 5000, 40000):
        for kind in range(4):
            b = rng.integers(0, 4, l_pac).astype(np.uint8)
            if kind == 1:
                b[:] = b[0]
            elif kind == 2:
                b = np.resize(rng.integers(0, 4, 7), l_pac).astype(np.uint8)
            elif kind == 3:
                b = np.resize(rng.integers(0, 4, max(1, l_pac // 10)), l_pac).astype(np.uint8)
                e = rng.random(l_pac) < 0.01
                b[e] = rng.integers(0, 4, int(e.sum()))
            pac = np.zeros((l_pac + 3) // 4, np.uint8)
            np.bitwise_or.at(pac, np.arange(l_pac) >> 2, (b << ((~np.arange(l_pac) & 3) << 1)).astype(np.uint8))
            text = np.concatenate([b, 3 - b[::-1]]).astype(np.uint8)
            n = len(text)
            sa = index.suffix_array(text).astype(np.int64)
            primary = int(np.nonzero(sa == 0)[0][0])
            sym = text[sa[sa != 0] - 1].astype(np.uint32)
            sym = np.concatenate([sym, np.zeros((-len(sym)) % 16, np.uint32)]).reshape(-1, 16)
            want = np.zeros(len(sym), np.uint32)
            for j in range(16):
                want |= sym[:, j] << np.uint32((15 - j) * 2)
            for intv in (1, 32):
                for chunk in (0, 300, 2000):
                    bwt = np.empty((n + 15) // 16, np.uint32)
                    samples = np.empty((n + intv) // intv, np.uint64)
                    pr = ctypes.c_uint64()
                    rc = gpu_ctx.L.bsb_build_bwt(gpu_ctx.handle, pac.ctypes.data_as(ctypes.c_void_p), l_pac, intv,
                                                 chunk, bwt.ctypes.data_as(ctypes.c_void_p), ctypes.byref(pr),
                                                 samples.ctypes.data_as(ctypes.c_void_p))
                    if rc == _lib.BSB_ENOMEM and chunk:
                        continue                     # a bucket larger than the chunk
                    _lib.check(gpu_ctx.handle, rc)
                    assert pr.value == primary, (l_pac, kind, chunk)
                    assert np.array_equal(bwt, want), (l_pac, kind, chunk)
                    assert np.array_equal(samples, sa[::intv].astype(np.uint64)), (l_pac, kind, chunk, intv)
