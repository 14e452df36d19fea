"""The integer form of the reference's band caps, (int)((double)num / e + 1.) at ksw.c:402,405,
bwamem.c:627-628 and bwa.c:234-235, which the CUDA kernels compute as (num + e) / e truncated
toward zero (band_cap, bsbolt_gb300/csrc/bsb_internal.cuh): equal over every numerator and gap
extension the kernels can meet, negative numerators included.  CPU only."""
import numpy as np


def test_band_cap_equals_double_form():
    num = np.arange(-200_000, 200_001, dtype=np.int64)
    for e in range(1, 65):
        ref = np.trunc(num.astype(np.float64) / e + 1.0).astype(np.int64)    # C's (int) truncates
        # C integer division of (num + e) by e, truncating toward zero
        q = np.abs(num + e) // e * np.sign(num + e)
        assert np.array_equal(ref, q), e
