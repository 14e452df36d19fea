"""Read sets and `bwa mem` runs shared by the SAM-identity tests (tests/test_bwa_glue.py on
the CPU, tests/test_bwa_gpu.py on the GPU).  Everything is seeded and synthetic."""
import os
import subprocess

import numpy as np

from bsbolt_gb300 import synth

# bsbolt Align's default `bwa mem` argv (bsbolt/Utils/Launcher.py:75-103 with the defaults of
# bsbolt/Utils/Parser.py:46-110), threads and -K fixed
BSBOLT_ARGS = ["-A", "1", "-B", "4", "-D", "0.5", "-E", "1,1", "-L", "30,30", "-T", "10", "-U", "17", "-W", "0",
               "-c", "500", "-d", "100", "-k", "19", "-m", "50", "-r", "1.5", "-w", "100", "-y", "20", "-O", "6,6",
               "-h", "100,200", "-e", "0.1", "-l", "0.5", "-n", "5", "-Z", "0.95"]


def write_fastq(path, reads, tag):
    letters = np.frombuffer(b"ACGTN", np.uint8)
    with open(path, "w") as f:
        for i, r in enumerate(reads):
            s = letters[r].tobytes().decode()
            f.write(f"@r{i}/{tag}\n{s}\n+\n{'?' * len(s)}\n")


def index(bwa, fa):
    subprocess.check_call([bwa, "index", "-a", "bwtsw", fa], stderr=subprocess.DEVNULL)


def pe_set(d, bwa):
    """3 x 200 kb bisulfite reference with a duplicated block; 3,000 directional 2 x 100 pairs,
    60 pairs whose one end only mate rescue places, 20 random pairs."""
    contigs = synth.bs_genome(3, 200_000, seed=4242)
    contigs[1][1][50_000:55_000] = contigs[0][1][10_000:15_000]      # a duplicated block
    fa = os.path.join(d, "ref.fa")
    synth.write_fasta(fa, contigs)
    index(bwa, fa)
    r1, r2 = synth.bs_reads_pe(contigs, 3000, 100, 300, 30, seed=4243)
    # pairs with one end mutated at every 10th base (by +1, which neither conversion
    # undoes): no exact 19-mer, so that end has no seed and only mate rescue places it
    m1, m2 = synth.bs_reads_pe(contigs, 60, 100, 300, 30, seed=4245)
    for k, (a, b) in enumerate(zip(m1, m2)):
        x = b if k % 2 == 0 else a
        x[5::10] = (x[5::10] + 1) % 4
    r1 += m1
    r2 += m2
    rng = np.random.Generator(np.random.PCG64(4244))
    for _ in range(20):
        r1.append(rng.integers(0, 4, 100).astype(np.uint8))
        r2.append(rng.integers(0, 4, 100).astype(np.uint8))
    write_fastq(os.path.join(d, "r1.fq"), r1, 1)
    write_fastq(os.path.join(d, "r2.fq"), r2, 2)
    # an undirectional library: half of the pairs come with their ends swapped, so read 1
    # carries the G->A pattern (bsbolt Align -UN, `bwa mem -z`)
    u1 = [b if k % 2 else a for k, (a, b) in enumerate(zip(r1, r2))]
    u2 = [a if k % 2 else b for k, (a, b) in enumerate(zip(r1, r2))]
    write_fastq(os.path.join(d, "u1.fq"), u1, 1)
    write_fastq(os.path.join(d, "u2.fq"), u2, 2)
    return fa, os.path.join(d, "r1.fq"), os.path.join(d, "r2.fq"), os.path.join(d, "u1.fq"), os.path.join(d, "u2.fq")


def long_set(d, bwa):
    """Reads the seed-level Smith-Waterman filter runs on (mem_flt_chained_seeds,
    bwamem.c:602-619): single-end reads of 513-1023 bases on the pe_set reference (at 5.5*ln(L)
    <= 0.05*L, i.e. from ~724 bases, the filter runs with -W 0), and 2 x 150 pairs for runs with
    -W (min_chain_weight), where it runs from 22*W bases.  Returns (fa, long.fq, p1.fq, p2.fq);
    pe_set must have been built in d."""
    contigs = synth.bs_genome(3, 200_000, seed=4242)
    contigs[1][1][50_000:55_000] = contigs[0][1][10_000:15_000]
    fa = os.path.join(d, "ref.fa")
    reads = []
    for k, L in enumerate((513, 600, 723, 724, 760, 900, 1023)):
        r1, _ = synth.bs_reads_pe(contigs, 60, L, L + 200, 20, seed=4260 + k)
        reads += r1
    write_fastq(os.path.join(d, "long.fq"), reads, 1)
    p1, p2 = synth.bs_reads_pe(contigs, 1500, 150, 400, 40, seed=4270)
    write_fastq(os.path.join(d, "p150_1.fq"), p1, 1)
    write_fastq(os.path.join(d, "p150_2.fq"), p2, 2)
    return fa, os.path.join(d, "long.fq"), os.path.join(d, "p150_1.fq"), os.path.join(d, "p150_2.fq")


def repeat_set(d, bwa, copies=700, n_pairs=40):
    """2 x 300 kb reference holding `copies` exact copies of one 300-base element, and read
    pairs from inside copies: every seed has more rows than max_occ (500), mem_chain samples
    500 of them (bwamem.c:281-283), and each read gets hundreds of regions -- more than the
    first guess of the glue's region buffer."""
    rng = np.random.Generator(np.random.PCG64(4250))
    contigs = synth.bs_genome(2, 300_000, seed=4251)
    elem = contigs[0][1][1000:1300].copy()
    slots = rng.permutation(np.arange(2, 2 * 290_000 // 400))[:copies]
    for s in slots:
        c = contigs[int(s) % 2][1]
        at = 400 * (int(s) // 2) + 2_000
        c[at:at + 300] = elem
    fa = os.path.join(d, "rep.fa")
    synth.write_fasta(fa, contigs)
    index(bwa, fa)
    # pairs from a fragment that lies wholly inside the element, so every copy matches
    r1, r2 = synth.bs_reads_pe([("elem", elem)], n_pairs, 100, 200, 20, seed=4252)
    write_fastq(os.path.join(d, "rep1.fq"), r1, 1)
    write_fastq(os.path.join(d, "rep2.fq"), r2, 2)
    return fa, os.path.join(d, "rep1.fq"), os.path.join(d, "rep2.fq")


def run_mem(binary, fa, reads, extra, env=None, threads=4):
    """SAM lines of `binary mem -Y -t threads -K 10000000 extra fa reads...`, without @PG
    (it carries argv[0])."""
    cmd = [binary, "mem", "-Y", "-t", str(threads), "-K", "10000000"] + extra + [fa] + list(reads)
    out = subprocess.run(cmd, capture_output=True, check=True, env=env).stdout.decode()
    return [line for line in out.splitlines() if not line.startswith("@PG")]


def run_stats(binary, fa, reads, extra, env_key, prefix):
    """stderr counters that the glue prints at exit: {name: (kept, served)} and regrown."""
    cmd = [binary, "mem", "-Y", "-t", "4", "-K", "10000000"] + extra + [fa] + list(reads)
    res = subprocess.run(cmd, capture_output=True, check=True, env=dict(os.environ, **{env_key: "1"}))
    stats = {}
    for line in res.stderr.decode().splitlines():
        if not line.startswith(prefix):
            continue
        w = line.split()
        if w[1] in ("cigar", "matesw"):
            stats[w[1]] = (int(w[4]), int(w[6]))
        elif w[1] == "region":
            stats["regrown"] = int(w[-1])
    return stats
