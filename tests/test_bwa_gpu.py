"""`bwa_gpu mem` -- BSBolt's BWA fork linked to libbsbgpu.so -- writes the stock `bwa mem`
SAM byte for byte, on the GPU.

bwa_gpu (bsbolt_gb300/integration/Makefile) is the reference's own sources, unmodified, with
its worker1 pass (seeds -> SA -> chains -> mem_chain2aln -> mem_sort_dedup_patch for the whole
-K batch), the bwa_gen_cigar2 calls of worker2 and the mate-rescue ksw_align2 calls served by
the CUDA library through link-time wraps (bwamem_gpu_hook.c).  The stock `bwa` is the same
sources built by oracle/Makefile.ref.  Every SAM line but @PG (it carries argv[0]) must be
identical: paired and single end, bsbolt Align's default command line, end bonus 5 and 30,
no mate rescue, two other scorings, an undirectional library (-z), and reads in a repeat
family larger than max_occ.  The GPU served counts show that the CUDA results, not the
reference's fallbacks, produced the SAM.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BWA = os.path.join(ROOT, "oracle", "_ref", "bwa")
GPU = os.path.join(ROOT, "bsbolt_gb300", "integration", "_build", "bwa_gpu")
STAGED = os.path.join(ROOT, "baseline", "_ref", "bwa", "bwamem.c")

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import sam_sets  # noqa: E402

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not os.path.exists(STAGED), reason="reference BWA sources not staged")]


@pytest.fixture(scope="module")
def pe(tmp_path_factory):
    # staged sources with no binaries means the build failed: that is an error, not a skip
    assert os.path.exists(BWA) and os.path.exists(GPU), "bwa / bwa_gpu were not built from the staged sources"
    return sam_sets.pe_set(str(tmp_path_factory.mktemp("gpu_sam")), BWA)


def same(fa, reads, extra, min_lines):
    ref = sam_sets.run_mem(BWA, fa, reads, extra)
    got = sam_sets.run_mem(GPU, fa, reads, extra)
    assert len(ref) >= min_lines
    if got != ref:
        bad = [k for k, (a, b) in enumerate(zip(got, ref)) if a != b][:3]
        raise AssertionError(f"{len(got)} vs {len(ref)} lines; first differences:\n" +
                             "\n".join(f"gpu: {got[k]}\nref: {ref[k]}" for k in bad))


ARGV = {
    "bsbolt_default": sam_sets.BSBOLT_ARGS,
    "bonus5": ["-A", "1", "-B", "4", "-O", "6,6", "-E", "1,1", "-L", "5,5", "-w", "100", "-d", "100"],
    "bonus30": ["-L", "30,30"],
    "no_rescue": ["-L", "5,5", "-S"],
    "scoring_a2": ["-A", "2", "-B", "5", "-O", "5,7", "-E", "2,1", "-L", "5,5"],
    "scoring_a3_word_lanes": ["-A", "3", "-B", "5", "-O", "6,6", "-E", "1,1", "-T", "60", "-L", "5,5"],
}


@pytest.mark.parametrize("name", list(ARGV))
def test_gpu_sam_paired_end(pe, name):
    fa, r1, r2 = pe[:3]
    same(fa, [r1, r2], ARGV[name], 6000)


def test_gpu_sam_single_end(pe):
    fa, r1 = pe[0], pe[1]
    same(fa, [r1], ["-L", "5,5"], 3000)
    same(fa, [r1], sam_sets.BSBOLT_ARGS, 3000)


def test_gpu_sam_undirectional(pe):
    fa, u1, u2 = pe[0], pe[3], pe[4]
    same(fa, [u1, u2], ["-z"] + sam_sets.BSBOLT_ARGS, 6000)


def test_gpu_results_are_served(pe):
    """The GPU CIGAR records and mate-rescue results answer worker2's calls: the SAM above
    comes from the CUDA library, not from the reference's own functions."""
    fa, r1, r2 = pe[:3]
    st = sam_sets.run_stats(GPU, fa, [r1, r2], ["-L", "5,5"], "BSB_GPU_STATS", "[bsb_gpu]")
    kept, served = st["cigar"]
    assert kept > 5000 and served > 0.9 * 6000, st
    assert st["matesw"][0] > 0 and st["matesw"][1] > 0, st


def test_gpu_repeat_family_over_max_occ(tmp_path):
    """700 exact copies of an element: ~500 regions per read, more than the glue's first
    region buffer; the library answers BSB_ECAPACITY, the batch runs again, SAM identical."""
    assert os.path.exists(BWA) and os.path.exists(GPU)
    fa, r1, r2 = sam_sets.repeat_set(str(tmp_path), BWA)
    same(fa, [r1, r2], ["-L", "5,5"], 80)
    same(fa, [r1, r2], sam_sets.BSBOLT_ARGS, 80)
    st = sam_sets.run_stats(GPU, fa, [r1, r2], ["-L", "5,5"], "BSB_GPU_STATS", "[bsb_gpu]")
    assert st["regrown"] >= 1, st


def test_gpu_long_reads_and_seed_sw_filter(pe):
    """Reads of 513-1023 bases and 2 x 150 pairs under -W 5: the seed-level Smith-Waterman
    filter (mem_flt_chained_seeds) runs on the GPU and the SAM is the reference's."""
    fa, lf, p1, p2 = sam_sets.long_set(os.path.dirname(pe[0]), BWA)
    same(fa, [lf], ["-L", "5,5"], 420)
    same(fa, [lf], sam_sets.BSBOLT_ARGS, 420)
    same(fa, [p1, p2], ["-W", "5", "-L", "5,5"], 3000)


@pytest.mark.parametrize("workers", ["2", "3", "5"])
def test_gpu_sam_many_batches_and_pipeline_workers(pe, workers):
    """-K 30000 cuts the pairs into ~20 batches; with 2 (the reference's, bwa_gpu's default), 3
    and 5 workers in mem's read -> align -> write pipeline the SAM is the stock one."""
    fa, r1, r2 = pe[:3]
    extra = sam_sets.BSBOLT_ARGS + ["-K", "30000"]
    ref = sam_sets.run_mem(BWA, fa, [r1, r2], extra)
    got = sam_sets.run_mem(GPU, fa, [r1, r2], extra, env=dict(os.environ, BSB_PIPELINE_WORKERS=workers))
    assert len(ref) > 6000 and got == ref
