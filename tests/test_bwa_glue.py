"""The BWA glue (bsbolt_gb300/integration/bwamem_gpu.c) produces the reference's SAM.

`oracle/_ref/bwa_glue` is the reference `bwa` (built from its own sources by
oracle/Makefile.ref) whose worker1 pass goes through mem_align_batch_gpu --
the glue a maintainer adds -- with the CPU oracle answering
bsb_align_regs_batch (on the GPU the library gives the same regions, by
tests/test_align_gpu.py).  Its `bwa mem` SAM must equal the stock `bwa mem`
SAM byte for byte (the @PG line carries argv[0] and is compared without it),
for directional paired-end bisulfite reads, with end bonus 5 and bsbolt's 30.
CPU only; skipped where the reference build is absent.
"""
import os
import subprocess

import numpy as np
import pytest

from bsbolt_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref")
BWA, GLUE = os.path.join(REF, "bwa"), os.path.join(REF, "bwa_glue")

pytestmark = pytest.mark.skipif(not (os.path.exists(BWA) and os.path.exists(GLUE)),
                                reason="reference bwa / bwa_glue not built here (oracle/Makefile.ref)")


def write_fastq(path, reads, tag):
    letters = np.frombuffer(b"ACGTN", np.uint8)
    with open(path, "w") as f:
        for i, r in enumerate(reads):
            s = letters[r].tobytes().decode()
            f.write(f"@r{i}/{tag}\n{s}\n+\n{'?' * len(s)}\n")


@pytest.fixture(scope="module")
def data(tmp_path_factory):
    d = tmp_path_factory.mktemp("glue")
    contigs = synth.bs_genome(3, 200_000, seed=4242)
    contigs[1][1][50_000:55_000] = contigs[0][1][10_000:15_000]      # a duplicated block
    fa = str(d / "ref.fa")
    synth.write_fasta(fa, contigs)
    subprocess.check_call([BWA, "index", "-a", "bwtsw", fa], stderr=subprocess.DEVNULL)
    r1, r2 = synth.bs_reads_pe(contigs, 3000, 100, 300, 30, seed=4243)
    # pairs with one end mutated at every 10th base (by +1, which neither conversion
    # undoes): no exact 19-mer, so that end has no seed and only mate rescue places it
    m1, m2 = synth.bs_reads_pe(contigs, 60, 100, 300, 30, seed=4245)
    for k, (a, b) in enumerate(zip(m1, m2)):
        x = b if k % 2 == 0 else a
        x[5::10] = (x[5::10] + 1) % 4
    r1 += m1
    r2 += m2
    # a few adapter-like / random / short reads
    rng = np.random.Generator(np.random.PCG64(4244))
    for _ in range(20):
        r1.append(rng.integers(0, 4, 100).astype(np.uint8))
        r2.append(rng.integers(0, 4, 100).astype(np.uint8))
    write_fastq(str(d / "r1.fq"), r1, 1)
    write_fastq(str(d / "r2.fq"), r2, 2)
    return fa, str(d / "r1.fq"), str(d / "r2.fq")


def run_mem(binary, fa, r1, r2, extra, env=None):
    cmd = [binary, "mem", "-Y", "-t", "4", "-K", "10000000"] + extra + [fa, r1, r2]
    out = subprocess.run(cmd, capture_output=True, check=True, env=env).stdout.decode()
    return [line for line in out.splitlines() if not line.startswith("@PG")]


@pytest.mark.parametrize("bonus", ["5,5", "30,30"])
def test_glue_sam_identical_to_reference(data, bonus):
    fa, r1, r2 = data
    extra = ["-A", "1", "-B", "4", "-O", "6,6", "-E", "1,1", "-L", bonus, "-w", "100", "-d", "100"]
    ref = run_mem(BWA, fa, r1, r2, extra)
    glue = run_mem(GLUE, fa, r1, r2, extra)
    assert len(ref) > 6000
    assert glue == ref


def test_glue_path_is_live(data):
    """Perturbing one region inside the glue path changes the SAM: the comparison above
    really runs through mem_align_batch_gpu."""
    fa, r1, r2 = data
    extra = ["-L", "5,5"]
    env = dict(os.environ, BSB_SHIM_PERTURB="1")
    assert run_mem(GLUE, fa, r1, r2, extra, env) != run_mem(BWA, fa, r1, r2, extra)


def test_glue_cigar_records_are_served(data):
    """The CIGAR pre-pass answers most of worker2's bwa_gen_cigar2 calls (the SAM above is
    identical with them), and a perturbed record reaches the SAM."""
    fa, r1, r2 = data
    extra = ["-L", "5,5"]
    cmd = [GLUE, "mem", "-Y", "-t", "4", "-K", "10000000"] + extra + [fa, r1, r2]
    res = subprocess.run(cmd, capture_output=True, check=True, env=dict(os.environ, BSB_SHIM_STATS="1"))
    line = [x for x in res.stderr.decode().splitlines() if x.startswith("[bsb_glue] cigar records")][-1]
    kept, served = int(line.split()[4]), int(line.split()[6])
    assert kept > 5000 and served > 0.9 * 6000, line
    env = dict(os.environ, BSB_SHIM_PERTURB_CIGAR="1")
    assert run_mem(GLUE, fa, r1, r2, extra, env) != run_mem(BWA, fa, r1, r2, extra)


def test_glue_matesw_results_are_served(data):
    """The mate-rescue pre-pass answers worker2's ksw_align2 calls from mem_matesw (the
    SAM of the identity test above is produced with them), and a perturbed result reaches
    the SAM."""
    fa, r1, r2 = data
    extra = ["-L", "5,5"]
    cmd = [GLUE, "mem", "-Y", "-t", "4", "-K", "10000000"] + extra + [fa, r1, r2]
    res = subprocess.run(cmd, capture_output=True, check=True, env=dict(os.environ, BSB_SHIM_STATS="1"))
    line = [x for x in res.stderr.decode().splitlines() if x.startswith("[bsb_glue] matesw jobs")][-1]
    kept, served = int(line.split()[4]), int(line.split()[6])
    assert kept > 0 and served > 0, line
    env = dict(os.environ, BSB_SHIM_PERTURB_SW="1")
    assert run_mem(GLUE, fa, r1, r2, extra, env) != run_mem(BWA, fa, r1, r2, extra)


def test_glue_single_end_identical(data):
    """Single-end reads (worker2 without pairing or mate rescue) through the glue: the same SAM."""
    fa, r1, _ = data
    extra = ["-L", "5,5"]
    cmd = ["-Y", "-t", "4", "-K", "10000000"] + extra + [fa, r1]
    ref = subprocess.run([BWA, "mem"] + cmd, capture_output=True, check=True).stdout.decode().splitlines()
    glue = subprocess.run([GLUE, "mem"] + cmd, capture_output=True, check=True).stdout.decode().splitlines()
    ref = [x for x in ref if not x.startswith("@PG")]
    glue = [x for x in glue if not x.startswith("@PG")]
    assert len(ref) > 3000 and glue == ref


def test_glue_without_mate_rescue(data):
    """`-S` (MEM_F_NO_RESCUE): the rescue pre-pass keeps nothing and the SAM stays the reference's."""
    fa, r1, r2 = data
    extra = ["-L", "5,5", "-S"]
    assert run_mem(GLUE, fa, r1, r2, extra) == run_mem(BWA, fa, r1, r2, extra)
    cmd = [GLUE, "mem", "-Y", "-t", "4", "-K", "10000000"] + extra + [fa, r1, r2]
    res = subprocess.run(cmd, capture_output=True, check=True, env=dict(os.environ, BSB_SHIM_STATS="1"))
    line = [x for x in res.stderr.decode().splitlines() if x.startswith("[bsb_glue] matesw jobs")][-1]
    assert int(line.split()[4]) == 0 and int(line.split()[6]) == 0, line


@pytest.mark.parametrize("scoring", [["-A", "2", "-B", "5", "-O", "5,7", "-E", "2,1"],
                                     ["-A", "3", "-B", "5", "-O", "6,6", "-E", "1,1", "-T", "60"]])
def test_glue_other_scorings(data, scoring):
    """Other scoring through every hook: with -A 3 a 100-base mate's rescue runs on word lanes
    (qlen * a >= 250) and the CIGAR band and dedup thresholds move."""
    fa, r1, r2 = data
    extra = scoring + ["-L", "5,5"]
    ref = run_mem(BWA, fa, r1, r2, extra)
    assert len(ref) > 6000 and run_mem(GLUE, fa, r1, r2, extra) == ref
