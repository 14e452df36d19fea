"""The suffix array sorted on the GPU (bsb_build_suffix_array, prefix doubling) gives the
reference `bwa index` files byte for byte (tests/golden/index*_sha256.json, which the
reference produced), and the host SA-IS order on texts with long repeats."""
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


@pytest.mark.parametrize("gen,fixture", [(golden_data.golden_genome, "index_sha256.json"),
                                         (golden_data.golden_genome_rep, "index_rep_sha256.json")],
                         ids=["plain", "repeats"])
def test_gpu_suffix_array_gives_reference_index_files(gpu_ctx, tmp_path, gen, fixture):
    fa = str(tmp_path / "ref.fa")
    synth.write_fasta(fa, gen())
    index.build_index(fa, str(tmp_path / "ref"), ctx=gpu_ctx)
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
