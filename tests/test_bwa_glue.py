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
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref")
BWA, GLUE = os.path.join(REF, "bwa"), os.path.join(REF, "bwa_glue")

pytestmark = pytest.mark.skipif(not (os.path.exists(BWA) and os.path.exists(GLUE)),
                                reason="reference bwa / bwa_glue not built here (oracle/Makefile.ref)")


sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import sam_sets  # noqa: E402


@pytest.fixture(scope="module")
def pe(tmp_path_factory):
    return sam_sets.pe_set(str(tmp_path_factory.mktemp("glue")), BWA)


@pytest.fixture(scope="module")
def data(pe):
    return pe[:3]


@pytest.fixture(scope="module")
def undirectional(pe):
    return pe[0], pe[3], pe[4]


def run_mem(binary, fa, r1, r2, extra, env=None):
    return sam_sets.run_mem(binary, fa, [r1, r2], extra, env)


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


def test_glue_bsbolt_default_argv(data):
    """bsbolt Align's own default `bwa mem` command line (-L 30,30, -T 10, the XA and
    bisulfite options)."""
    fa, r1, r2 = data
    ref = run_mem(BWA, fa, r1, r2, sam_sets.BSBOLT_ARGS)
    assert len(ref) > 6000 and run_mem(GLUE, fa, r1, r2, sam_sets.BSBOLT_ARGS) == ref


def test_glue_undirectional(undirectional):
    """`-z` (bsbolt Align -UN): ambiguous pairs are aligned under both conversions
    (bwa.c:95-133), and the glue sees the duplicated reads as any others."""
    fa, u1, u2 = undirectional
    extra = ["-z", "-L", "5,5"]
    ref = run_mem(BWA, fa, u1, u2, extra)
    assert len(ref) > 6000 and run_mem(GLUE, fa, u1, u2, extra) == ref


def test_glue_repeat_family_over_max_occ(tmp_path):
    """Reads inside a family of 700 exact copies: each has ~500 regions (max_occ rows
    sampled per seed), more than the glue's first region buffer holds; the library
    answers BSB_ECAPACITY with the size it needs, the batch runs again, and the SAM is the
    reference's."""
    fa, r1, r2 = sam_sets.repeat_set(str(tmp_path), BWA)
    extra = ["-L", "5,5"]
    ref = run_mem(BWA, fa, r1, r2, extra)
    assert len(ref) >= 80 and run_mem(GLUE, fa, r1, r2, extra) == ref
    st = sam_sets.run_stats(GLUE, fa, [r1, r2], extra, "BSB_SHIM_STATS", "[bsb_glue]")
    assert st["regrown"] >= 1, st


def test_glue_long_reads_and_seed_sw_filter(pe):
    """Reads of 513-1023 bases (the seed-level SW filter of mem_flt_chained_seeds runs from ~724)
    and 2 x 150 pairs under -W 5 (the filter runs on every read): the glue's regions and the
    reference's SAM agree."""
    fa, lf, p1, p2 = sam_sets.long_set(os.path.dirname(pe[0]), BWA)
    for extra in (["-L", "5,5"], sam_sets.BSBOLT_ARGS):
        ref = sam_sets.run_mem(BWA, fa, [lf], extra)
        assert len(ref) >= 420 and sam_sets.run_mem(GLUE, fa, [lf], extra) == ref
    extra = ["-W", "5", "-L", "5,5"]
    ref = run_mem(BWA, fa, p1, p2, extra)
    assert len(ref) >= 3000 and run_mem(GLUE, fa, p1, p2, extra) == ref


def _records(path):
    with open(path) as f:
        lines = f.read().splitlines()
    return [lines[i:i + 4] for i in range(0, len(lines), 4)]


def _write(path, recs, eol="\n", final_eol=True, blank_after=None, header=None, fasta=False, opener=open):
    out = []
    for k, r in enumerate(recs):
        h = header(k, r[0]) if header else r[0]
        if fasta:
            s = r[1]
            out += [">" + h[1:]] + [s[i:i + 60] for i in range(0, len(s), 60)]
        else:
            out += [h, r[1], "+", r[3]]
        if blank_after is not None and k == blank_after:
            out.append("")
    text = eol.join(out) + (eol if final_eol else "")
    with opener(path, "wt") as f:
        f.write(text)


@pytest.mark.parametrize("variant", ["comments", "double_readno_undirectional", "crlf", "fasta_multiline",
                                     "blank_line", "no_final_newline", "gzip", "small_batches_se_undirectional"])
def test_glue_fastq_reader_matches_kseq(pe, tmp_path, variant):
    """bwa_glue reads its input with the glue's FASTQ reader (bseq_fast.c: a line scan and entries
    built on threads, the reference's bseq_read for anything else); the SAM must equal the stock
    reader's for headers with comments (-C copies them into the SAM), names ending in /1/2 under
    -z (bseq_read trims a duplicated read's name twice), CRLF line ends, multi-line FASTA, a blank
    line between records, a file without its last newline, gzip input, and many small batches."""
    import gzip
    fa, r1, r2 = pe[:3]
    a, b = _records(r1)[:1500], _records(r2)[:1500]
    p1, p2 = str(tmp_path / "a.fq"), str(tmp_path / "b.fq")
    extra = ["-L", "5,5"]
    if variant == "comments":
        hdr = lambda k, h: f"{h}\tBC:Z:ACGT{k % 7}  x"          # noqa: E731
        _write(p1, a, header=hdr)
        _write(p2, b, header=hdr)
        extra += ["-C"]
    elif variant == "double_readno_undirectional":
        hdr = lambda k, h: h[:-2] + "/7" + h[-2:]                # noqa: E731  r1/7/1: trimmed to r1/7, then r1
        _write(p1, a, header=hdr)
        _write(p2, b, header=hdr)
        extra += ["-z"]
    elif variant == "crlf":
        _write(p1, a, eol="\r\n")
        _write(p2, b, eol="\r\n")
    elif variant == "fasta_multiline":
        _write(p1, a, fasta=True)
        _write(p2, b, fasta=True)
    elif variant == "blank_line":
        _write(p1, a, blank_after=900)
        _write(p2, b, blank_after=900)
    elif variant == "no_final_newline":
        _write(p1, a, final_eol=False)
        _write(p2, b, final_eol=False)
    elif variant == "gzip":
        p1, p2 = p1 + ".gz", p2 + ".gz"
        _write(p1, a, opener=gzip.open)
        _write(p2, b, opener=gzip.open)
    else:
        _write(p1, a + b)
        p2 = None
        extra += ["-z", "-K", "20000"]
    reads = [p1] + ([p2] if p2 else [])
    ref = sam_sets.run_mem(BWA, fa, reads, extra)
    glue = sam_sets.run_mem(GLUE, fa, reads, extra)
    assert len(ref) >= 3000 and glue == ref


def _bsstat(binary, fa, reads, extra):
    cmd = [binary, "mem", "-Y", "-t", "4", "-K", "200000"] + extra + [fa] + list(reads)
    err = subprocess.run(cmd, capture_output=True, check=True).stderr.decode()
    tot = {}
    for line in err.splitlines():
        if line.startswith("BSStat "):
            k, v = line.split()[1:3]
            tot[k] = tot.get(k, 0) + int(v)
    return tot


@pytest.mark.parametrize("mode", ["pe", "se", "se_undirectional"])
def test_glue_output_step_bsstat_matches_samsorter(pe, mode):
    """The glue's output step (sam_out.c, in place of samSorter) prints the same BSStat counts
    per batch as the reference's samSorter -- summed over many small batches (-K 200000) -- for
    pairs, single ends, and -z, whose ambiguous reads take the unmapped rewrite."""
    fa, r1, r2 = pe[:3]
    reads = [r1, r2] if mode == "pe" else [r1]
    extra = ["-L", "5,5"] + (["-z"] if mode == "se_undirectional" else [])
    ref = _bsstat(BWA, fa, reads, extra)
    glue = _bsstat(GLUE, fa, reads, extra)
    assert ref and glue == ref
    if mode == "se_undirectional":
        assert ref["BSAmbiguous:"] > 0


def test_glue_reads_string_by_string(pe):
    """With BSB_SAM_WRITER=0 the FASTQ reader allocates every read's strings one by one (the
    reference's samSorter frees them so); the glue's output step then frees them one by one as
    well, in many small batches, and the SAM is the stock one."""
    fa, r1, r2 = pe[:3]
    extra = ["-L", "5,5", "-K", "50000"]
    ref = sam_sets.run_mem(BWA, fa, [r1, r2], extra)
    glue = sam_sets.run_mem(GLUE, fa, [r1, r2], extra, env=dict(os.environ, BSB_SAM_WRITER="0"))
    assert len(ref) >= 3000 and glue == ref
