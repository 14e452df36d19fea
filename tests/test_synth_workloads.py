"""The synthetic workload generators the bench's configurations rest on (CPU only)."""
import numpy as np

from bsbolt_gb300 import synth


def test_rrbs_reads_start_at_mspi_fragment_ends():
    """Every RRBS-like read is a prefix of an MspI fragment (C^CGG cut, 40-220 bases) on one of
    its strands, 75 or 100 bases long or the fragment if shorter; before conversion and errors
    the first bases are the cut site's CGG (top strand) or the fragment's far end (bottom)."""
    contigs = synth.bs_genome(2, 600_000, seed=31)
    frags = synth.rrbs_fragments(contigs)
    assert len(frags) > 10
    for k, a, b in frags:
        g = contigs[k][1]
        assert 40 <= b - a <= 220
        assert list(g[a - 1:a + 3]) == [1, 1, 2, 2] and list(g[b - 1:b + 3]) == [1, 1, 2, 2]
    seqs, offs = synth.rrbs_reads_se(contigs, 5000, meth_cpg=1.0, meth_ch=1.0, err=0.0, seed=32)
    lens = np.diff(offs)
    assert len(lens) == 5000 and lens.min() >= 40 and lens.max() <= 100
    assert ((lens == 75) | (lens == 100)).mean() > 0.5      # the rest: fragments shorter than the read
    starts = set()
    for k, a, b in frags:
        f = contigs[k][1][a:b]
        for s in (f, synth.COMP[f[::-1]]):
            starts.add(bytes(s[:40]))
    # with every C methylated and no errors the reads are exact fragment prefixes
    assert all(bytes(seqs[offs[i]:offs[i] + 40]) in starts for i in range(0, 5000, 7))
    # few fragments, many reads: heavy duplication of start positions
    assert len({bytes(seqs[offs[i]:offs[i] + 40]) for i in range(5000)}) <= 2 * len(frags)


def test_matesw_jobs_shapes():
    jobs, seq = synth.matesw_jobs(300, seed=5)
    assert (jobs["qlen"] >= 30).all() and (jobs["qlen"] <= 250).all()
    assert (jobs["tlen"] >= jobs["qlen"] + 20).all()
    assert (jobs["qoff"] + jobs["qlen"] <= len(seq)).all() and (jobs["toff"] + jobs["tlen"] <= len(seq)).all()
    byte = (jobs["xtra"] & 0x10000) != 0
    assert np.array_equal(byte, jobs["qlen"] < 250)
