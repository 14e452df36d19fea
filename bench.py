#!/usr/bin/env python
"""Benchmark: batched ksw_extend2 (the extension half of BSBolt's bisulfite
seed-extend path) on one GB300, plain schedule.

Workload (N=1 line): 4,000,000 extension jobs -- query length U[10,140] in the
three-letter converted alphabet (A/G/T ~ 30/20/50 %, 1 % N), target = query
with 1 % substitutions and 0.1 % indels (1-5 nt) plus 100 nt of flank, 20 %
unrelated targets, h0 ~ U[19,100], w = 100, BWA default scoring (a=1, b=4,
o=6, e=1, z-drop 100, end bonus 5).  Seeded synthetic data (numpy PCG64).

value  = GCUPS with every input resident in HBM, cells = the reference cell
         count (sum over rows of end-beg of ksw_extend2's own loop),
         device time from CUDA events on the library's stream.
e2e    = GCUPS through the C ABI bsb_extend_batch with pinned host buffers:
         H2D of jobs + sequences, kernels, D2H of the tuples, every step.
roofline = integer pipe: 14 int ops per reference cell against the measured
         add+max throughput of this GPU for the cell width the dominant kernel
         computes in (bsb_probe_int16x2_peak for the 16-bit two-cells-per-register
         kernels of even-C shapes, bsb_probe_int_peak for the 32-bit ones).
cpu_baseline = the reference's own ksw_extend2, compiled from BSBolt's sources
         (oracle/_ref/libref_ksw.so), on a bounded sample, all host cores.

--impl reference: the same reference ksw_extend2 timed on the host cores over
the workload, all cores (the oracle port of ksw.c:380-479 when the reference
sources were not staged).
Further blocks of the same JSON line (each skippable): the seeds -> regions
pass on a 2 Mb, a 100 Mb (PE and RRBS-like) and the 3.1 Gb human-scale
reference (index sorted on the GPU), the learned job and read orders, the tile
autotuner, bwa_gen_cigar2, mate rescue, and stock bwa mem against bwa_gpu mem
from SAM.
Multi-GPU: replicas only -- every rank extends its own 4M-job batch.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "extension GCUPS (batched ksw_extend2, plain schedule)"
UNIT = "GCUPS"
INT_OPS_PER_CELL = 14          # add+select, 2 max, select+max, 2x(sub, max0, sub, max): ksw.c:431-447
SCHED_KERNELS = 3              # schedule: hist, scan, scatter (then the persistent kernels of each tile shape:
                               # 16-bit cells + the 32-bit kernel for jobs over the 16-bit limit when C is even,
                               # the 32-bit kernel alone when C is odd)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def rank_seed(rank):
    """Each replica extends its own batch: the 4M-job workload's generator seed, offset by rank."""
    return 20261203 + 1 + rank


def replica_totals(elapsed, cells, dist=None, device="cpu"):
    """Whole-job figures of a replicas run (no data-path collective): the slowest rank's
    time and the cells of every rank.  Without a process group, this rank's own figures."""
    if dist is None:
        return float(elapsed), float(cells)
    import torch
    t = torch.tensor([float(elapsed)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor([float(cells)], device=device, dtype=torch.float64)
    dist.all_reduce(c)
    return float(t.item()), float(c.item())


def cached_jobs(n, seed):
    from bsbolt_gb300 import synth
    d = os.path.join(tempfile.gettempdir(), "bsbgpu_cache")
    os.makedirs(d, exist_ok=True)
    fj = os.path.join(d, f"jobs_{n}_{seed}.npy")
    fs = os.path.join(d, f"seq_{n}_{seed}.npy")
    if os.path.exists(fj) and os.path.exists(fs):
        try:
            return np.load(fj).view(synth.JOB_DTYPE).reshape(-1), np.load(fs)
        except Exception:
            pass
    jobs, seq = synth.ksw_jobs(n, seed=seed)
    np.save(fj + ".tmp.npy", jobs.view(np.uint8).reshape(len(jobs), -1))
    np.save(fs + ".tmp.npy", seq)
    os.replace(fj + ".tmp.npy", fj)
    os.replace(fs + ".tmp.npy", fs)
    return jobs, seq


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        self.out.flush()
        rows = []
        try:
            with open(self.out.name) as f:
                for line in f:
                    parts = [p.strip() for p in line.split(",")]
                    if len(parts) >= 9:
                        rows.append(parts)
        finally:
            os.unlink(self.out.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_port_gcups(jobs, seq, n_sample, threads, mat):
    import oracle
    sub = jobs[:n_sample]
    t0 = time.perf_counter()
    out, cells = oracle.ksw_batch(sub, seq, mat, 6, 1, 6, 1, 100, n_threads=threads)
    dt = time.perf_counter() - t0
    return float(cells.sum()) / dt / 1e9, dt, out, cells


_SAMPLE_CELLS = {}


def cpu_reference_gcups(jobs, seq, n_sample, threads, mat):
    """The reference's own compiled ksw_extend2 (oracle/_ref/libref_ksw.so) on the first
    n_sample jobs over `threads` host threads, when the reference sources were staged and
    built; else the C port (oracle/bsb_oracle.c).  The sample's cell count comes from the
    port (once, untimed): the reference does not report it.  Returns (GCUPS, seconds, tuples,
    cells, kind)."""
    import oracle
    if not oracle.have_reference_ksw():
        g, dt, out, cells = cpu_port_gcups(jobs, seq, n_sample, threads, mat)
        return g, dt, out, cells, "port"
    sub = jobs[:n_sample]
    key = (id(jobs), n_sample)
    if key not in _SAMPLE_CELLS:
        _SAMPLE_CELLS[key] = oracle.ksw_batch(sub, seq, mat, 6, 1, 6, 1, 100, n_threads=threads)[1]
    cells = _SAMPLE_CELLS[key]
    t0 = time.perf_counter()
    out = oracle.ref_ksw_batch(sub, seq, mat, 6, 1, 6, 1, 100, n_threads=threads)
    dt = time.perf_counter() - t0
    return float(cells.sum()) / dt / 1e9, dt, out, cells, "reference"


def ref2mb_workload(n_pairs=20000):
    """The 2 Mb-reference workload: 4 x 500 kb reference (GC 41 %, CpG 1 %), directional PE 2x100,
    insert N(300,30), CpG meth 0.8, CH 0.01, 99.5 % conversion, 0.5 % errors; the reads
    converted in silico as bsbolt does (read 1 C->T, read 2 G->A).  Cached on disk."""
    from bsbolt_gb300 import index, synth
    d = os.path.join(tempfile.gettempdir(), "bsbgpu_cache", f"ref2mb_{n_pairs}")
    os.makedirs(d, exist_ok=True)
    prefix = os.path.join(d, "ref")
    if not os.path.exists(prefix + ".sa") or not os.path.exists(os.path.join(d, "oreads.npy")):
        contigs = synth.bs_genome(4, 500_000, gc=0.41, cpg_frac=0.01, seed=20261203)
        synth.write_fasta(prefix + ".fa", contigs)
        index.build_index(prefix + ".fa", prefix)
        r1, r2 = synth.bs_reads_pe(contigs, n_pairs, 100, 300, 30, seed=20261203)
        reads, oreads = [], []
        for a, b in zip(r1, r2):
            reads.append(synth.bs_convert(a, g2a=False))
            reads.append(synth.bs_convert(b, g2a=True))
            oreads += [a, b]
        offs = np.zeros(len(reads) + 1, np.int64)
        offs[1:] = np.cumsum([len(r) for r in reads])
        np.save(os.path.join(d, "reads.npy"), np.concatenate(reads))
        np.save(os.path.join(d, "oreads.npy"), np.concatenate(oreads))
        np.save(os.path.join(d, "offs.npy"), offs)
    return prefix, np.load(os.path.join(d, "reads.npy")), np.load(os.path.join(d, "offs.npy"))


def ref2mb_original_reads(n_pairs=20000):
    """The 2 Mb workload's reads as sequenced (before the in-silico conversion), same offsets."""
    ref2mb_workload(n_pairs)
    return np.load(os.path.join(tempfile.gettempdir(), "bsbgpu_cache", f"ref2mb_{n_pairs}", "oreads.npy"))


def infer_bw(l1, l2, score, a, q, r):
    """infer_bw (bwamem.c:796-803), vectorised; the double is truncated as C converts it."""
    l1, l2, score = (np.asarray(v, np.int64) for v in (l1, l2, score))
    w = np.trunc((np.minimum(l1, l2) * a - score - q) / r + 2.0).astype(np.int64)
    w = np.maximum(w, np.abs(l1 - l2))
    return np.where((l1 == l2) & (l1 * a - score < ((q + r - a) << 1)), 0, w)


def cigar_jobs_from_regions(regs, roff, offs, opt):
    """One bwa_gen_cigar2 job per read -- its best region, with the first band mem_reg2aln
    tries (bwamem.c:1219-1228): query = read + qb, the original read from its start."""
    n = len(roff) - 1
    has = np.nonzero(roff[1:] > roff[:-1])[0]
    best = np.array([roff[r] + int(np.argmax(regs["score"][roff[r]:roff[r + 1]])) for r in has], np.int64)
    g = regs[best]
    l1, l2 = g["qe"] - g["qb"], g["re"] - g["rb"]
    w2 = np.maximum(infer_bw(l1, l2, g["truesc"], opt.a, opt.o_del, opt.e_del),
                    infer_bw(l1, l2, g["truesc"], opt.a, opt.o_ins, opt.e_ins))
    w2 = np.where(w2 > opt.w, np.minimum(w2, g["w"]), w2)
    w2 = np.minimum(w2, opt.w << 2)
    from bsbolt_gb300 import cigar
    jobs = np.zeros(len(best), cigar.JOB_DTYPE)
    jobs["rb"], jobs["re"] = g["rb"], g["re"]
    jobs["qoff"] = offs[has] + g["qb"]
    jobs["ooff"] = offs[has]
    jobs["l_query"] = l1
    jobs["w"] = w2
    return jobs, n


def matesw_block(ctx, steps, n_jobs=40000):
    """Mate-rescue Smith-Waterman (ksw_align2 as mem_matesw calls it): GPU batch through
    the C ABI (host buffers, copies included) against the CPU oracle on all host threads."""
    import oracle
    from bsbolt_gb300 import matesw, synth
    jobs, seq = synth.matesw_jobs(n_jobs)
    mat = synth.fill_scmat(1, 4)
    out = matesw.align2_batch(ctx, jobs, seq, mat, 6, 1, 6, 1)                # warm-up
    k = max(3, min(steps, 10))
    t0 = time.perf_counter()
    for _ in range(k):
        out = matesw.align2_batch(ctx, jobs, seq, mat, 6, 1, 6, 1)
    gpu_s = (time.perf_counter() - t0) / k
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ref = oracle.align2_batch(jobs, seq, mat, 6, 1, 6, 1, n_threads=threads)
    cpu_s = time.perf_counter() - t0
    same = bool(all(np.array_equal(out[f], ref[f]) for f in ref.dtype.names))
    # cells of the forward pass as the reference computes them: padded query columns x target rows
    p = np.where(jobs["xtra"] & matesw.KSW_XBYTE, 16, 8)
    cells = float(((jobs["qlen"] + p - 1) // p * p).astype(np.float64) @ jobs["tlen"].astype(np.float64))
    # the same job mix in a ten times larger batch (GPU only): throughput once the longest
    # jobs no longer set the batch time
    big, bseq = synth.matesw_jobs(10 * n_jobs, seed=20261203 + 6)
    matesw.align2_batch(ctx, big, bseq, mat, 6, 1, 6, 1)
    t0 = time.perf_counter()
    for _ in range(k):
        matesw.align2_batch(ctx, big, bseq, mat, 6, 1, 6, 1)
    big_s = (time.perf_counter() - t0) / k
    return {
        "workload": f"{n_jobs} ksw_align2 jobs shaped like mem_matesw's: mate of 30-250 bases vs a window of "
                    "read length + 20-700 bases (4 in 5 holding a mutated copy), KSW_XSUBO|KSW_XSTART|19, "
                    "byte lanes when qlen < 250, BWA scoring",
        "jobs": n_jobs, "forward_pass_cells": int(cells),
        "gpu_jobs_per_s": round(n_jobs / gpu_s, 1), "gpu_ms_per_batch": round(gpu_s * 1e3, 3),
        "gpu_forward_gcups": round(cells / gpu_s / 1e9, 2),
        "h2d_bytes_per_batch": int(jobs.nbytes + len(seq)), "d2h_bytes_per_batch": int(out.nbytes),
        "cpu_oracle_jobs_per_s": round(n_jobs / cpu_s, 1), "cpu_oracle_threads": threads,
        "cpu_oracle_note": "scalar restatement of the striped SSE2 code (oracle/bsb_oracle_sw.c), slower than "
                           "the reference's own SIMD build, which does not run on this Arm host",
        "results_bit_exact_vs_oracle": same,
        "gpu_jobs_per_s_batch_of_%d" % (10 * n_jobs): round(10 * n_jobs / big_s, 1),
    }


def cigar_block(ctx, steps):
    """bwa_gen_cigar2 for the best region of every read of the 2 Mb workload: GPU batch
    (host buffers, copies included) against the CPU oracle on all host threads."""
    import oracle
    from bsbolt_gb300 import _lib, cigar, index, seed, synth
    prefix, reads, offs = ref2mb_workload()
    oreads = ref2mb_original_reads()
    seed.load_index(ctx, prefix)
    bi = index.BwaIndex(prefix)
    opt = _lib.AlignOpt.bwa_defaults()
    regs, roff = seed.align_regs(ctx, reads, offs, opt)
    jobs, n_reads = cigar_jobs_from_regions(regs, roff, offs, opt)
    out, blob = cigar.gen_cigar_batch(ctx, jobs, reads, oreads, bi.crick_l, opt)        # warm-up
    k = max(3, min(steps, 10))
    t0 = time.perf_counter()
    for _ in range(k):
        out, blob = cigar.gen_cigar_batch(ctx, jobs, reads, oreads, bi.crick_l, opt)
    gpu_s = (time.perf_counter() - t0) / k
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ref, rblob = oracle.gen_cigar_batch(synth.fill_scmat(opt.a, opt.b), opt.o_del, opt.e_del, opt.o_ins, opt.e_ins,
                                        bi.l_pac, bi.pac, bi.opac, bi.crick_l, jobs, reads, oreads, n_threads=threads)
    cpu_s = time.perf_counter() - t0
    same = bool(all(np.array_equal(out[f], ref[f]) for f in ref.dtype.names if f != "pad")
                and np.array_equal(blob, rblob))
    n = len(jobs)
    return {
        "workload": "2 Mb bisulfite reference, the best region of each of the 40k reads of the 20k-pair "
                    "2x100 workload, first band of mem_reg2aln (infer_bw), bwa_gen_cigar2 as mem_reg2aln calls it",
        "jobs": n, "gapped_jobs": int((jobs["w"] > 0).sum()), "mean_band_w": round(float(jobs["w"].mean()), 2),
        "gpu_alignments_per_s": round(n / gpu_s, 1), "gpu_ms_per_batch": round(gpu_s * 1e3, 3),
        "h2d_bytes_per_batch": int(jobs.nbytes + reads.nbytes + oreads.nbytes),
        "d2h_bytes_per_batch": int(out.nbytes + len(blob)),
        "cpu_oracle_alignments_per_s": round(n / cpu_s, 1), "cpu_oracle_threads": threads,
        "records_bit_exact_vs_oracle": same,
        "status_counts": {str(s): int(c) for s, c in enumerate(np.bincount(out["status"], minlength=5))},
    }


def ref100mb_contigs():
    """The 100 Mb reference: 4 x 25 Mb (GC 41 %, CpG 1 %) with 15 % interspersed repeats of
    300 bp - 6 kb families at 2-15 % divergence."""
    from bsbolt_gb300 import synth
    contigs = synth.bs_genome(4, 25_000_000, gc=0.41, cpg_frac=0.01, seed=20261203 + 2)
    return synth.add_repeats(contigs, 0.15, seed=20261203 + 2)


def ref100mb_workload(n_pairs=100_000):
    """The 100 Mb-reference workload: 4 x 25 Mb reference (GC 41 %, CpG 1 %, 15 % interspersed
    repeats of 300 bp - 6 kb families at 2-15 % divergence), directional PE 2x150, insert
    N(400,50), the 2 Mb workload's methylation/conversion/error model.  Cached on disk."""
    from bsbolt_gb300 import index, synth
    d = os.path.join(tempfile.gettempdir(), "bsbgpu_cache", f"ref100mb_{n_pairs}")
    os.makedirs(d, exist_ok=True)
    prefix = os.path.join(d, "ref")
    if not os.path.exists(os.path.join(d, "offs.npy")):
        contigs = ref100mb_contigs()
        if not os.path.exists(prefix + ".sa"):
            synth.write_fasta(prefix + ".fa", contigs)
            index.build_index(prefix + ".fa", prefix)
        r1, r2 = synth.bs_reads_pe_block(contigs, n_pairs, 150, 400, 50, seed=20261203 + 2)
        r1 = synth.bs_convert(r1, g2a=False)          # the aligner's in-silico conversion
        r2 = synth.bs_convert(r2, g2a=True)
        reads = np.stack([r1, r2], axis=1).reshape(-1)
        offs = np.arange(2 * n_pairs + 1, dtype=np.int64) * 150
        np.save(os.path.join(d, "reads.npy"), reads)
        np.save(os.path.join(d, "offs.npy"), offs)
    return prefix, np.load(os.path.join(d, "reads.npy")), np.load(os.path.join(d, "offs.npy"))


def rrbs_workload(n_reads=3_000_000):
    """The RRBS-like workload on the 100 Mb reference: directional single-end reads, half 1x75 and
    half 1x100, starting at the ends of MspI fragments of 40-220 bases (so heavily duplicated),
    CpG methylation 0.7.  Cached on disk beside the 100 Mb index."""
    from bsbolt_gb300 import synth
    prefix, _, _ = ref100mb_workload()
    d = os.path.dirname(prefix)
    fr, fo = os.path.join(d, f"rrbs_{n_reads}.npy"), os.path.join(d, f"rrbs_{n_reads}_offs.npy")
    if not os.path.exists(fo):
        seqs, offs = synth.rrbs_reads_se(ref100mb_contigs(), n_reads, seed=20261203 + 3)
        conv = seqs.copy()
        conv[conv == 1] = 3                     # the aligner's C->T conversion of read 1 (bs_helpers.cpp:18-31)
        np.save(fr, conv)
        np.save(fo, offs)
    return prefix, np.load(fr), np.load(fo)


def pipeline_rrbs(ctx, batch_bases=10_000_000, cpu_reads=4_000):
    """bsb_mem_align1_batch on the RRBS-like workload in -K 10M-base batches, against the CPU
    oracle (chains, extension and mem_sort_dedup_patch) on a sample."""
    import oracle
    from bsbolt_gb300 import _lib, index, seed
    t0 = time.perf_counter()
    prefix, reads, offs = rrbs_workload()
    prep_s = time.perf_counter() - t0
    n_reads = len(offs) - 1
    seed.load_index(ctx, prefix)
    opt = _lib.AlignOpt.bwa_defaults()
    batches, lo = [], 0
    while lo < n_reads:                        # -K: reads until the batch holds batch_bases bases
        hi = int(np.searchsorted(offs, offs[lo] + batch_bases, side="left"))
        hi = max(lo + 1, min(hi, n_reads))
        batches.append((lo, hi))
        lo = hi

    def sub(a, b):
        return reads[offs[a]:offs[b]], offs[a:b + 1] - offs[a]
    seed.align_regs(ctx, *sub(*batches[0]), opt, dedup=True)     # warm-up
    t0 = time.perf_counter()
    first = None
    stages = dict.fromkeys(seed.ALIGN_STAGES, 0.0)
    for a, b in batches:
        regs, roff = seed.align_regs(ctx, *sub(a, b), opt, dedup=True)
        add_stages(stages, ctx)
        if first is None:
            first = (regs, roff)
    gpu_s = time.perf_counter() - t0
    bi = index.BwaIndex(prefix)
    ob = oracle.OracleBwt(bi.primary, bi.L2[1:], bi.bwt, bi.sa, bi.sa_intv)
    anns = np.array([(a.offset, a.len, 0) for a in bi.anns], dtype=oracle.ANN_DTYPE)
    threads = os.cpu_count() or 1
    cr, co = sub(0, cpu_reads)
    oo = oracle.Opt.from_list([1, 4, 6, 1, 6, 1, 100, 100, 5, 5, 19, 500, 10, 20, 10000])
    t0 = time.perf_counter()
    pre = oracle.align_regs(ob, anns, bi.pac, bi.l_pac, oo, cr, co, n_threads=threads)
    ref, ref_off = oracle.sort_dedup_batch(oo, bi.l_pac, bi.pac, cr, co, pre["regs"], pre["regs_off"])
    cpu_s = time.perf_counter() - t0
    regs, roff = first
    k = int(roff[cpu_reads])
    exact = bool(np.array_equal(roff[:cpu_reads + 1], ref_off) and
                 all(np.array_equal(regs[f][:k], ref[f]) for f in ref.dtype.names))
    lens = np.diff(offs)
    return {
        "workload": f"RRBS-like: {n_reads} directional single-end reads (1x75 and 1x100, shorter where the fragment is) "
                    "starting at the ends of MspI fragments of 40-220 bases of the 100 Mb reference, CpG methylation "
                    f"0.7, -K 10M-base batches ({len(batches)}), BWA defaults",
        "stage": "bsb_mem_align1_batch (seeds -> ... -> mem_sort_dedup_patch), host buffers incl. H2D/D2H",
        "gpu_reads_per_s": round(n_reads / gpu_s, 1),
        "gpu_ms_per_batch": round(gpu_s / len(batches) * 1e3, 3),
        "mean_read_len": round(float(lens.mean()), 1),
        "cpu_oracle_reads_per_s": round(cpu_reads / cpu_s, 1),
        "cpu_oracle_threads": threads, "cpu_sample_reads": cpu_reads,
        "regions_bit_exact_vs_oracle_on_sample": exact,
        "workload_prep_s": round(prep_s, 1),
        "stage_ms_per_batch": {k: round(v / len(batches), 3) for k, v in stages.items()},
    }


def measured_hbm_gbs():
    """HBM copy bandwidth of this GPU pool (MEASURED_PEAKS.json, written per machine), else the
    fallback figure."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def seeding_roofline(ctx, reads, offs, reps=5):
    """Device time of one seeding batch (seed_kernel's two launches, the offset scan and the
    compaction: bsb_seed_batch_device) with CUDA events on the context stream, and the
    occurrence-query bytes it reads as algorithmic traffic: per bwt_extend one bwt_2occ4 =
    two queries, 32 B each in the device's sector layout (64 B each in the reference's
    128-symbol blocks)."""
    import ctypes
    import torch
    from bsbolt_gb300 import _lib, seed
    n = len(offs) - 1
    total = int(offs[-1] - offs[0])
    d_reads = torch.from_numpy(np.ascontiguousarray(reads[offs[0]:offs[-1]])).cuda()
    d_offs = torch.from_numpy(np.ascontiguousarray(offs - offs[0])).cuda()
    d_out = torch.empty((2 * total + 32 * n) * 4, dtype=torch.int64, device="cuda")
    d_off = torch.empty(n + 1, dtype=torch.int64, device="cuda")
    opt = _lib.SeedOpt(19, 1.5, 10, 20)
    max_len = int(np.diff(offs).max())

    def launch():
        _lib.check(ctx.handle, ctx.L.bsb_seed_batch_device(ctx.handle, ctypes.byref(opt), n,
                                                           ctypes.c_void_p(d_reads.data_ptr()),
                                                           ctypes.c_void_p(d_offs.data_ptr()), total, max_len,
                                                           ctypes.c_void_p(d_out.data_ptr()),
                                                           ctypes.c_void_p(d_off.data_ptr())))
    s = torch.cuda.ExternalStream(ctx.stream)
    for _ in range(2):
        launch()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s)
    for _ in range(reps):
        launch()
    b.record(s)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / reps
    n_ext = seed.last_extensions(ctx)
    seeds = int(d_off[-1].item())
    peak, src = measured_hbm_gbs()
    bytes32 = n_ext * 2 * 32
    gbs = bytes32 / (ms * 1e-3) / 1e9
    return {"reads": n, "seeds": seeds, "bwt_extend_calls": n_ext, "occ_queries": 2 * n_ext,
            "ms_per_batch": round(ms, 4), "seeds_per_s": round(seeds / (ms * 1e-3), 1),
            "reads_per_s": round(n / (ms * 1e-3), 1),
            "algorithmic_bytes_sector_layout": bytes32, "algorithmic_bytes_reference_layout": 2 * bytes32,
            "achieved_gbs": round(gbs, 2), "peak_gbs": peak, "frac": round(gbs / peak, 4),
            "frac_reference_layout_bytes": round(2 * gbs / peak, 4),
            "peak_source": f"HBM copy bandwidth, {src} (MEASURED_PEAKS.json hbm_gbs)"}


def add_stages(acc, ctx):
    """Adds the last alignment batch's device ms per stage (bsb_last_stage_ms) to acc."""
    from bsbolt_gb300 import seed
    for k, v in seed.last_stage_ms(ctx).items():
        acc[k] += v


def pipeline_ref100mb(ctx, batch_pairs=33_333, cpu_pairs=2_000):
    """Seeds -> regions on the 100 Mb reference (200 MB BWT, larger than L2) in -K 10M-base
    batches, against the CPU oracle on a sample."""
    import oracle
    from bsbolt_gb300 import _lib, index, seed
    t0 = time.perf_counter()
    prefix, reads, offs = ref100mb_workload()
    prep_s = time.perf_counter() - t0
    n_reads = len(offs) - 1
    seed.load_index(ctx, prefix)
    opt = _lib.AlignOpt.bwa_defaults()
    b = 2 * batch_pairs
    batches = [(lo, min(n_reads, lo + b)) for lo in range(0, n_reads, b)]

    def sub(lo, hi):
        return reads[offs[lo]:offs[hi]], offs[lo:hi + 1] - offs[lo]
    seed.align_regs(ctx, *sub(*batches[0]))                      # warm-up
    t0 = time.perf_counter()
    first = None
    stages = dict.fromkeys(seed.ALIGN_STAGES, 0.0)
    for lo, hi in batches:
        regs, roff = seed.align_regs(ctx, *sub(lo, hi))
        add_stages(stages, ctx)
        if first is None:
            first = (regs, roff)
    gpu_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    for lo, hi in batches:
        seed.seed_batch(ctx, *sub(lo, hi))
    seed_s = time.perf_counter() - t0
    lo, hi = batches[0]
    seeding = seeding_roofline(ctx, reads, offs[lo:hi + 1])
    bi = index.BwaIndex(prefix)
    ob = oracle.OracleBwt(bi.primary, bi.L2[1:], bi.bwt, bi.sa, bi.sa_intv)
    anns = np.array([(a.offset, a.len, 0) for a in bi.anns], dtype=oracle.ANN_DTYPE)
    threads = os.cpu_count() or 1
    cr, co = sub(0, 2 * cpu_pairs)
    t0 = time.perf_counter()
    ref = oracle.align_regs(ob, anns, bi.pac, bi.l_pac,
                            oracle.Opt.from_list([1, 4, 6, 1, 6, 1, 100, 100, 5, 5, 19, 500, 10, 20, 10000]),
                            cr, co, n_threads=threads)
    cpu_s = time.perf_counter() - t0
    regs, roff = first
    k = int(roff[2 * cpu_pairs])
    exact = bool(np.array_equal(roff[:2 * cpu_pairs + 1], ref["regs_off"]) and
                 all(np.array_equal(regs[f][:k], ref["regs"][f]) for f in ("rb", "re", "qb", "qe", "score", "truesc")))
    n_pairs = n_reads // 2
    return {
        "workload": "100 Mb bisulfite reference (4x25 Mb, 15% interspersed repeats, BWT 200 MB > L2), "
                    f"{n_pairs} directional PE 2x150 pairs in -K 10M-base batches of {batch_pairs} pairs, BWA defaults",
        "gpu_read_pairs_per_s": round(n_pairs / gpu_s, 1),
        "gpu_ms_per_batch": round(gpu_s / len(batches) * 1e3, 3),
        "gpu_seeding_reads_per_s": round(n_reads / seed_s, 1),
        "cpu_oracle_read_pairs_per_s": round(cpu_pairs / cpu_s, 1),
        "cpu_oracle_threads": threads, "cpu_sample_pairs": cpu_pairs,
        "regions_bit_exact_vs_oracle_on_sample": exact,
        "workload_prep_s": round(prep_s, 1),
        "stage_ms_per_batch": {k: round(v / len(batches), 3) for k, v in stages.items()},
        "seeding_roofline_one_batch": seeding,
    }


def sam_sha(path):
    """SHA-256 of a SAM file without its @PG line (which carries argv[0]), and its line count."""
    import hashlib
    h, n = hashlib.sha256(), 0
    with open(path, "rb") as f:
        for line in f:
            if not line.startswith(b"@PG"):
                h.update(line)
                n += 1
    return h.hexdigest(), n


def time_bwa_mem(binary, db, fastqs, threads, out_sam, env=None):
    """Wall time of `binary mem` with bsbolt Align's default argv (bsbolt_gb300.align) at
    -t threads and -K 10000000, SAM to out_sam; returns (seconds, BSStat counts)."""
    from bsbolt_gb300 import align
    cmd = align.bwa_command(binary, db, fastqs[0], fastqs[1] if len(fastqs) > 1 else None, t=threads)
    t0 = time.perf_counter()
    lines = []
    with open(out_sam, "wb") as f:
        stats = align.run_alignment(cmd, f, ["-K", "10000000"], env=env, echo=False, keep=lines)
    return time.perf_counter() - t0, stats, [x for x in lines if x.startswith("[bsb_gpu]")]


def bsbolt_db(prefix):
    """A bsbolt database directory (<db>/BSB_ref.fa.*, the layout `bsbolt Align -DB` reads)
    whose files link to the index at prefix."""
    db = prefix + "_bsbdb"
    os.makedirs(db, exist_ok=True)
    for ext in ("bwt", "sa", "pac", "opac", "ann", "amb"):
        link = os.path.join(db, "BSB_ref.fa." + ext)
        if not os.path.lexists(link):
            os.symlink(os.path.abspath(prefix + "." + ext), link)
    return db


def sam_workloads(n_pairs_100mb, n_rrbs):
    """FASTQ files of the SAM-level runs: the 2 Mb workload's 20k 2x100 pairs (as sequenced),
    n_pairs_100mb 2x150 pairs on the 100 Mb reference (insert N(400,50)) and n_rrbs RRBS-like
    single-end reads on it.  Cached on disk beside the indexes (whose files the bwa binaries read:
    they are byte-identical to the reference `bwa index`'s)."""
    from bsbolt_gb300 import synth
    out = {}
    prefix2, _, offs2 = ref2mb_workload()
    d2 = os.path.dirname(prefix2)
    if not os.path.exists(os.path.join(d2, "r2.fq")):
        o = ref2mb_original_reads().reshape(-1, 100)
        synth.write_fastq_block(os.path.join(d2, "r1.fq"), o[0::2], 1)
        synth.write_fastq_block(os.path.join(d2, "r2.fq"), o[1::2], 2)
    out["pe_2mb"] = (bsbolt_db(prefix2), [os.path.join(d2, "r1.fq"), os.path.join(d2, "r2.fq")], (len(offs2) - 1) // 2)
    if n_pairs_100mb or n_rrbs:
        prefix, _, _ = ref100mb_workload()
        d = os.path.dirname(prefix)
        contigs = None
        if n_pairs_100mb:
            f1, f2 = (os.path.join(d, f"pe150_{n_pairs_100mb}_{k}.fq") for k in (1, 2))
            if not os.path.exists(f2):
                contigs = contigs or ref100mb_contigs()
                r1, r2 = synth.bs_reads_pe_block(contigs, n_pairs_100mb, 150, 400, 50, seed=20261203 + 2 + 100)
                synth.write_fastq_block(f1, r1, 1)
                synth.write_fastq_block(f2 + ".tmp", r2, 2)
                os.replace(f2 + ".tmp", f2)
            out["pe_100mb"] = (bsbolt_db(prefix), [f1, f2], n_pairs_100mb)
        if n_rrbs:
            f1 = os.path.join(d, f"rrbs_{n_rrbs}.fq")
            if not os.path.exists(f1):
                contigs = contigs or ref100mb_contigs()
                seqs, offs = synth.rrbs_reads_se(contigs, n_rrbs, seed=20261203 + 3)
                synth.write_fastq_ragged(f1 + ".tmp", seqs, offs, 1)
                os.replace(f1 + ".tmp", f1)
            out["rrbs_100mb"] = (bsbolt_db(prefix), [f1], n_rrbs)
    return out


def sam_compare(name, db, fqs, n_units, threads):
    """One workload through the stock `bwa mem` and `bwa_gpu mem`: wall times, SAM and BSStat
    identity, and bwa_gpu's own account of its time."""
    stock = os.path.join(ROOT, "oracle", "_ref", "bwa")
    gpu = os.path.join(ROOT, "bsbolt_gb300", "integration", "_build", "bwa_gpu")
    tmp = os.path.join(tempfile.gettempdir(), "bsbgpu_cache", "sam")
    os.makedirs(tmp, exist_ok=True)
    sam_r, sam_g = os.path.join(tmp, name + ".ref.sam"), os.path.join(tmp, name + ".gpu.sam")
    tr, st_r, _ = time_bwa_mem(stock, db, fqs, threads, sam_r)
    tg, st_g, glog = time_bwa_mem(gpu, db, fqs, threads, sam_g, dict(os.environ, BSB_GPU_STATS="1"))
    hr, nr = sam_sha(sam_r)
    hg, ng = sam_sha(sam_g)
    for f in (sam_r, sam_g):
        os.unlink(f)
    unit = "read pairs" if len(fqs) == 2 else "reads"
    u = unit.replace(" ", "_")
    return {unit: n_units, "sam_lines": nr,
            f"stock_bwa_{u}_per_s": round(n_units / tr, 1), "stock_bwa_s": round(tr, 3),
            f"bwa_gpu_{u}_per_s": round(n_units / tg, 1), "bwa_gpu_s": round(tg, 3),
            "speedup": round(tr / tg, 3), "sam_identical": bool(hr == hg and nr == ng),
            "bsstat_identical": st_r == st_g, "bsstat": st_g, "bwa_gpu_log": glog}


def sam_block(n_pairs_100mb=500_000, n_rrbs=1_000_000, threads=None):
    """Aligned read pairs/s from SAM: the stock `bwa mem` (the reference BWA fork built from its
    own sources, oracle/Makefile.ref) against `bwa_gpu mem` (the same sources linked to
    libbsbgpu.so), both with bsbolt Align's default argv, -t = all host cores, -K 10000000, on
    the same FASTQ; the two SAM files must be identical but for @PG."""
    stock = os.path.join(ROOT, "oracle", "_ref", "bwa")
    gpu = os.path.join(ROOT, "bsbolt_gb300", "integration", "_build", "bwa_gpu")
    if not (os.path.exists(stock) and os.path.exists(gpu)):
        return {"error": "bwa / bwa_gpu not built (the reference sources were not staged)"}
    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    wl = sam_workloads(n_pairs_100mb, n_rrbs)
    prep_s = time.perf_counter() - t0
    res = {"argv": "bsbolt Align defaults (-Y -A1 -B4 -O6,6 -E1,1 -L30,30 -T10 -U17 -w100 -d100 -k19 -c500 "
                   "-h100,200 -e0.1 -l0.5 -n5 -Z0.95 ...) -t %d -K 10000000" % threads,
           "threads": threads, "workload_prep_s": round(prep_s, 1)}
    for name, (db, fqs, n_units) in wl.items():
        res[name] = sam_compare(name, db, fqs, n_units, threads)
    return res


ADAPTER1 = "AGATCGGAAGAGCACACGTCTGAACTCCAGTCACATCACGATCTCGTATGCCGTCTTCTGCTTGAAAAAAAAAA"


def ref1gb_reads(contigs, n_pairs, seed):
    """The human-scale workload's read mix, scaled: 70 % 2x150 (insert N(400,50)) and 30 % 2x250
    (insert N(550,60)) directional pairs; in 2 % of the pairs the fragment is shorter than the
    read and the read runs into adapter.  Returns [(r1, r2)] per read length, bases as sequenced."""
    from bsbolt_gb300 import synth
    ad = synth.NT4[np.frombuffer(ADAPTER1.encode(), np.uint8)]
    out = []
    rng = np.random.Generator(np.random.PCG64(seed))
    for k, (rl, frac, ins, sd) in enumerate(((150, 0.7, 400, 50), (250, 0.3, 550, 60))):
        r1, r2 = synth.bs_reads_pe_block(contigs, int(n_pairs * frac), rl, ins, sd, seed=seed + 1 + k)
        for j in np.nonzero(rng.random(len(r1)) < 0.02)[0]:
            c = int(rng.integers(rl // 2, rl))                 # fragment length below the read length
            frag = r1[j, :c].copy()
            r1[j, c:] = np.resize(ad, rl - c)
            r2[j, :c] = synth.COMP[frag[::-1]]
            r2[j, c:] = np.resize(ad[::-1], rl - c)
        out.append((r1, r2))
    return out


def human_contigs(tag):
    """The human-scale references: "1gb", 8 contigs of 125 Mb; "3gb", 24 contigs of 250 down to
    50 Mb (3.1 Gb); GC 41 %, CpG 1 %, 45 % interspersed repeats (families 300 bp - 6 kb, 2-20 %
    divergence)."""
    from bsbolt_gb300 import synth
    if tag == "1gb":
        contigs = synth.bs_genome(8, 125_000_000, gc=0.41, cpg_frac=0.01, seed=20261203 + 4)
    else:
        x = np.linspace(1.0, 0.0, 24) ** 1.53
        lens = np.round(50e6 + 200e6 * x).astype(np.int64)
        lens[0] += 3_100_000_000 - int(lens.sum())           # the total, on the longest contig
        assert 50e6 <= lens.min() and lens.max() <= 250e6
        contigs = []
        for k, ln in enumerate(lens):
            (_, g), = synth.bs_genome(1, int(ln), gc=0.41, cpg_frac=0.01, seed=20261203 + 300 + k)
            contigs.append((f"chr{k + 1}", g))
    synth.add_repeats(contigs, 0.45, fam_len=(300, 6000), div=(0.02, 0.20), n_families=500, seed=20261203 + 4)
    return contigs


def pipeline_ref1gb(ctx, n_pairs=200_000, batch_bases=10_000_000, tag="1gb", learned=False):
    """The human-scale configuration: a 1 Gb or the 3.1 Gb reference of human_contigs.  The index
    is built with the suffixes sorted on the GPU (bsb_build_bwt: 64-bit ranks, the 3.1 Gb text
    has 12.4e9 symbols with both conversions and strands) and held in HBM (occurrence sectors,
    full SA); then seeding's roofline on one -K batch, the regions pass (bsb_mem_align1_batch) over
    every pair, parity against the oracle on a sample, with `learned` the learned read order
    against the plain one (learned_order_compare, trained on the first quarter of the batches),
    and stock bwa against bwa_gpu from SAM."""
    import oracle
    from bsbolt_gb300 import _lib, index, seed, synth
    res = {}
    d = os.path.join(tempfile.gettempdir(), "bsbgpu_cache", "ref" + tag)
    os.makedirs(d, exist_ok=True)
    prefix = os.path.join(d, "ref")
    t0 = time.perf_counter()
    contigs = human_contigs(tag)
    res["genome_s"] = round(time.perf_counter() - t0, 1)
    if not os.path.exists(prefix + ".sa"):
        t0 = time.perf_counter()
        synth.write_fasta(prefix + ".fa", contigs)
        res["fasta_write_s"] = round(time.perf_counter() - t0, 1)
        t0 = time.perf_counter()
        res["index_build"] = index.build_index(prefix + ".fa", prefix, ctx=ctx)
        res["index_build_s"] = round(time.perf_counter() - t0, 1)
        os.unlink(prefix + ".fa")
    sets = ref1gb_reads(contigs, n_pairs, 20261203 + 40)
    del contigs
    fq = []
    for k, (r1, r2) in enumerate(sets):
        for e, r in ((1, r1), (2, r2)):
            fn = os.path.join(d, f"pe{k}_{e}.fq")
            synth.write_fastq_block(fn, r, e, first=sum(len(x[0]) for x in sets[:k]))
            fq.append(fn)
    for e in (1, 2):                                   # one FASTQ per end, both read lengths
        with open(os.path.join(d, f"r{e}.fq"), "wb") as f:
            for k in range(len(sets)):
                with open(os.path.join(d, f"pe{k}_{e}.fq"), "rb") as g:
                    f.write(g.read())
    t0 = time.perf_counter()
    seed.load_index(ctx, prefix)
    res["index_upload_s"] = round(time.perf_counter() - t0, 1)
    # the reads as the aligner sees them: read 1 C->T, read 2 G->A, pairs interleaved
    reads, lens = [], []
    for r1, r2 in sets:
        c1, c2 = synth.bs_convert(r1, g2a=False), synth.bs_convert(r2, g2a=True)
        reads.append(np.stack([c1, c2], axis=1).reshape(-1))
        lens.append(np.full(2 * len(r1), r1.shape[1], np.int64))
    reads = np.concatenate(reads)
    offs = np.zeros(sum(len(x) for x in lens) + 1, np.int64)
    offs[1:] = np.cumsum(np.concatenate(lens))
    n_reads = len(offs) - 1
    opt = _lib.AlignOpt.bwa_defaults()
    batches, lo = [], 0
    while lo < n_reads:
        hi = int(np.searchsorted(offs, offs[lo] + batch_bases, side="left"))
        hi = max(lo + 2, min(hi + (hi - lo) % 2, n_reads))
        batches.append((lo, hi))
        lo = hi

    def sub(a, b):
        return reads[offs[a]:offs[b]], offs[a:b + 1] - offs[a]
    res["seeding_roofline_one_batch"] = seeding_roofline(ctx, reads, offs[batches[0][0]:batches[0][1] + 1])
    seed.align_regs(ctx, *sub(*batches[0]), opt, dedup=True)       # warm-up
    t0 = time.perf_counter()
    first = None
    stages = dict.fromkeys(seed.ALIGN_STAGES, 0.0)
    for a, b in batches:
        regs, roff = seed.align_regs(ctx, *sub(a, b), opt, dedup=True)
        add_stages(stages, ctx)
        if first is None:
            first = (regs, roff)
    gpu_s = time.perf_counter() - t0
    bi = index.BwaIndex(prefix)
    ob = oracle.OracleBwt(bi.primary, bi.L2[1:], bi.bwt, bi.sa, bi.sa_intv)
    anns = np.array([(a.offset, a.len, 0) for a in bi.anns], dtype=oracle.ANN_DTYPE)
    oo = oracle.Opt.from_list([1, 4, 6, 1, 6, 1, 100, 100, 5, 5, 19, 500, 10, 20, 10000])
    ns = 1000
    cr, co = sub(0, ns)
    t0 = time.perf_counter()
    pre = oracle.align_regs(ob, anns, bi.pac, bi.l_pac, oo, cr, co, n_threads=os.cpu_count() or 1)
    ref, ref_off = oracle.sort_dedup_batch(oo, bi.l_pac, bi.pac, cr, co, pre["regs"], pre["regs_off"])
    cpu_s = time.perf_counter() - t0
    regs, roff = first
    k = int(roff[ns])
    exact = bool(np.array_equal(roff[:ns + 1], ref_off) and all(np.array_equal(regs[f][:k], ref[f])
                                                                  for f in ref.dtype.names))
    res.update({
        "workload": ("1 Gb bisulfite reference (8x125 Mb" if tag == "1gb" else
                     "3.1 Gb bisulfite reference (24 contigs of 250-50 Mb") +
                    f", 45% repeats), {n_reads // 2} directional pairs: 70% 2x150, "
                    f"30% 2x250, 2% adapter read-through; -K 10M batches ({len(batches)}); BWA defaults",
        "seq_len": int(bi.l_pac) * 2,
        "occ_layout": ("64-symbol sectors (0.5 B/row)" if os.environ.get("BSB_OCC_SYM64") == "1"
                       else "32-symbol sectors (1 B/row)"),
        "gpu_mem_align1_read_pairs_per_s": round(n_reads / 2 / gpu_s, 1),
        "cpu_oracle_read_pairs_per_s": round(ns / 2 / cpu_s, 1), "cpu_oracle_sample_reads": ns,
        "regions_bit_exact_vs_oracle_on_sample": exact})
    del bi, ob
    if learned:
        res["learned_read_order"] = learned_order_compare(
            ctx, reads, offs, batches, max(1, len(batches) // 4),
            f"{res['workload'].split(',')[0]}, {n_reads} reads in {len(batches)} -K 10M batches")
    threads = os.cpu_count() or 1
    if os.path.exists(os.path.join(ROOT, "bsbolt_gb300", "integration", "_build", "bwa_gpu")):
        # this process's full SA leaves the device first: bwa_gpu uploads the index again
        _lib.check(ctx.handle, ctx.L.bsb_index_full_sa(ctx.handle, 0))
        res["sam"] = sam_compare("pe_" + tag, bsbolt_db(prefix), [os.path.join(d, "r1.fq"), os.path.join(d, "r2.fq")],
                                 n_reads // 2, threads)
    return res


def learned_pipeline(ctx, batch_bases=10_000_000, train_batches=6):
    """The learned read order of the alignment batches against the plain (chain-count) order on
    the RRBS-like workload (learned_order_compare)."""
    from bsbolt_gb300 import seed
    prefix, reads, offs = rrbs_workload()
    n_reads = len(offs) - 1
    seed.load_index(ctx, prefix)
    batches, lo = [], 0
    while lo < n_reads:
        hi = int(np.searchsorted(offs, offs[lo] + batch_bases, side="left"))
        hi = max(lo + 1, min(hi, n_reads))
        batches.append((lo, hi))
        lo = hi
    return learned_order_compare(ctx, reads, offs, batches, train_batches,
                                 f"RRBS-like, {n_reads} reads in {len(batches)} -K 10M batches")


def learned_order_compare(ctx, reads, offs, batches, train_batches, label):
    """Per-read features and DP cells logged by the library from the first batches train the
    2x64 cost model on the GPU (bsb_mlp_* kernels); then every batch runs with the plain
    (chain-count), the learned and the exact-cost read order through bsb_mem_align1_batch (host
    buffers), regions compared.  The index is the one loaded."""
    import torch
    from bsbolt_gb300 import _lib, cost_model as cm, seed
    n_reads = int(batches[-1][1] - batches[0][0])
    opt = _lib.AlignOpt.bwa_defaults()

    def sub(a, b):
        return reads[offs[a]:offs[b]], offs[a:b + 1] - offs[a]
    # training logs: the first batches; evaluation logs: the last one
    seed.read_cost_log(ctx, True)
    feats, cells = [], []
    for a, b in batches[:train_batches] + [batches[-1]]:
        seed.align_regs(ctx, *sub(a, b), opt, dedup=True)
        f, c = seed.last_read_costs(ctx, b - a)
        feats.append(f)
        cells.append(c)
    seed.read_cost_log(ctx, False)
    ftr, ctr = np.concatenate(feats[:-1]), np.concatenate(cells[:-1])
    fev, cev = feats[-1], cells[-1]
    t0 = time.perf_counter()
    model = cm.CostModel(ctx, seed=5)
    losses = model.train(torch.from_numpy(ftr).cuda(), torch.from_numpy(np.log1p(ctr).astype(np.float32)).cuda(),
                         epochs=8)
    train_s = time.perf_counter() - t0
    pred = model.forward(torch.from_numpy(fev).cuda()).cpu().numpy()

    # every batch's logged cells: the keys of the exact-cost order (what a perfect model
    # would predict), which bounds the gain of any learned order
    seed.read_cost_log(ctx, True)
    exact_keys = []
    for a, b in batches:
        seed.align_regs(ctx, *sub(a, b), opt, dedup=True)
        exact_keys.append(seed.last_read_costs(ctx, b - a)[1])
    seed.read_cost_log(ctx, False)

    def run_all(exact=False):
        out, stages = [], dict.fromkeys(seed.ALIGN_STAGES, 0.0)
        t = time.perf_counter()
        for k, (a, b) in enumerate(batches):
            if exact:
                seed.set_read_order_keys(ctx, exact_keys[k])
            out.append(seed.align_regs(ctx, *sub(a, b), opt, dedup=True))
            for key, v in seed.last_stage_ms(ctx).items():
                stages[key] += v
        return time.perf_counter() - t, out, stages
    def with_model(m):
        seed.set_read_cost_model(ctx, m)
        try:
            return run_all()
        finally:
            seed.set_read_cost_model(ctx, None)
    run_all()                                      # warm-up of the three orders
    with_model(model)
    run_all(exact=True)
    # plain, learned, exact, twice: each order's time is the mean of its two passes, so a
    # drift of the GPU or the host over the runs falls on all alike
    runs = [run_all(), with_model(model), run_all(exact=True), run_all(), with_model(model), run_all(exact=True)]
    plain_out, learned_out, exact_out = runs[0][1], runs[1][1], runs[2][1]
    plain_s = (runs[0][0] + runs[3][0]) / 2
    learned_s = (runs[1][0] + runs[4][0]) / 2
    exact_s = (runs[2][0] + runs[5][0]) / 2
    plain_st = {k: (runs[0][2][k] + runs[3][2][k]) / 2 for k in seed.ALIGN_STAGES}
    learned_st = {k: (runs[1][2][k] + runs[4][2][k]) / 2 for k in seed.ALIGN_STAGES}
    exact_st = {k: (runs[2][2][k] + runs[5][2][k]) / 2 for k in seed.ALIGN_STAGES}
    # Amdahl: the read order changes only the chain2aln stage, so even a zero-time chain2aln
    # caps the gain at total / (total - chain2aln)
    tot = sum(plain_st.values())
    cap = tot / max(tot - plain_st["chain2aln"], 1e-9)
    same = all(np.array_equal(x[1], y[1]) and np.array_equal(x[0], y[0]) and np.array_equal(x[1], z[1]) and
               np.array_equal(x[0], z[0]) for x, y, z in zip(plain_out, learned_out, exact_out))
    # the plain order's key: chains per read (feature 1 is log1p(kept chains) / 4)
    plain_key = np.expm1(fev[:, 1] * 4)
    return {
        "workload": f"{label} (bsb_mem_align1_batch, host buffers)",
        "model": "2x64 MLP, BF16 weights, FP32 accumulation, per-read features (read length, kept chains, their "
                 "seeds, best chain weight, mean seed offset, reverse-strand share, C+G content, plain bound)",
        "trained_on": f"{len(ftr)} reads of the first {train_batches} batches, target log1p(DP cells) logged by "
                      "chain2aln_kernel", "train_s": round(train_s, 2),
        "train_loss_per_epoch": [round(x, 4) for x in losses],
        "spearman_model_eval_batch": round(cm.spearman(pred, cev), 4),
        "spearman_chain_count_eval_batch": round(cm.spearman(plain_key, cev), 4),
        "plain_reads_per_s": round(n_reads / plain_s, 1), "learned_reads_per_s": round(n_reads / learned_s, 1),
        "plain_s": round(plain_s, 4), "learned_s": round(learned_s, 4),
        "speedup_learned_vs_plain": round(plain_s / learned_s, 4), "regions_identical": bool(same),
        "stage_ms_all_batches": {"plain": {k: round(v, 2) for k, v in plain_st.items()},
                                 "learned": {k: round(v, 2) for k, v in learned_st.items()}},
        "chain2aln_share_plain": round(plain_st["chain2aln"] / max(tot, 1e-9), 4),
        "chain2aln_speedup_learned_vs_plain": round(plain_st["chain2aln"] / max(learned_st["chain2aln"], 1e-9), 4),
        "exact_cost_order": {"reads_per_s": round(n_reads / exact_s, 1), "s": round(exact_s, 4),
                             "speedup_vs_plain": round(plain_s / exact_s, 4),
                             "chain2aln_speedup_vs_plain": round(plain_st["chain2aln"] /
                                                                 max(exact_st["chain2aln"], 1e-9), 4),
                             "stage_ms_all_batches": {k: round(v, 2) for k, v in exact_st.items()}},
        "max_gain_from_any_read_order": round(cap, 4),
    }


def pipeline_secondary(ctx, steps, rank):
    """Seeds -> chains -> regions on the 2 Mb-reference workload, GPU vs the CPU oracle."""
    import oracle
    from bsbolt_gb300 import _lib, index, seed
    prefix, reads, offs = ref2mb_workload()
    n_pairs = (len(offs) - 1) // 2
    seed.load_index(ctx, prefix)
    opt = _lib.AlignOpt.bwa_defaults()
    regs, roff = seed.align_regs(ctx, reads, offs, opt)          # warm-up
    t0 = time.perf_counter()
    k = max(3, min(steps, 10))
    for _ in range(k):
        regs, roff = seed.align_regs(ctx, reads, offs, opt)
    gpu_s = (time.perf_counter() - t0) / k
    seed.seed_batch(ctx, reads, offs)
    t0 = time.perf_counter()
    for _ in range(k):
        sd, soff = seed.seed_batch(ctx, reads, offs)
    seed_s = (time.perf_counter() - t0) / k
    # the whole of mem_align1_core (with mem_sort_dedup_patch): bsb_mem_align1_batch
    dregs, droff = seed.align_regs(ctx, reads, offs, opt, dedup=True)
    t0 = time.perf_counter()
    for _ in range(k):
        dregs, droff = seed.align_regs(ctx, reads, offs, opt, dedup=True)
    full_s = (time.perf_counter() - t0) / k
    bi = index.BwaIndex(prefix)
    ob = oracle.OracleBwt(bi.primary, bi.L2[1:], bi.bwt, bi.sa, bi.sa_intv)
    anns = np.array([(a.offset, a.len, 0) for a in bi.anns], dtype=oracle.ANN_DTYPE)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ref = oracle.align_regs(ob, anns, bi.pac, bi.l_pac,
                            oracle.Opt.from_list([1, 4, 6, 1, 6, 1, 100, 100, 5, 5, 19, 500, 10, 20, 10000]),
                            reads, offs, n_threads=threads)
    oo = oracle.Opt.from_list([1, 4, 6, 1, 6, 1, 100, 100, 5, 5, 19, 500, 10, 20, 10000])
    cpu_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    dref, dref_off = oracle.sort_dedup_batch(oo, bi.l_pac, bi.pac, reads, offs, ref["regs"], ref["regs_off"])
    cpu_dedup_s = time.perf_counter() - t0
    exact = bool(np.array_equal(roff, ref["regs_off"]) and
                 all(np.array_equal(regs[f], ref["regs"][f]) for f in ("rb", "re", "qb", "qe", "score", "truesc")))
    dexact = bool(np.array_equal(droff, dref_off) and
                  all(np.array_equal(dregs[f], dref[f]) for f in dref.dtype.names))
    return {
        "workload": "2 Mb bisulfite reference (4x500 kb), 20k directional PE 2x100 pairs, "
                    "BWA defaults, -L 5",
        "stage": "seeds -> SA -> chains -> chain filter -> mem_chain2aln (pre-dedup regions, bsb_align_regs_batch, "
                 "host buffers incl. H2D/D2H)",
        "gpu_read_pairs_per_s": round(n_pairs / gpu_s, 1),
        "gpu_ms_per_batch": round(gpu_s * 1e3, 3),
        "gpu_seeding_reads_per_s": round(2 * n_pairs / seed_s, 1),
        "seeds_per_batch": int(soff[-1]),
        "cpu_oracle_read_pairs_per_s": round(n_pairs / cpu_s, 1),
        "cpu_oracle_threads": threads,
        "regions_bit_exact_vs_oracle": exact,
        "regions": int(roff[-1]),
        "ext_cells": int(ref["cells"]),
        "mem_align1_stage": "the same plus mem_sort_dedup_patch per read (bsb_mem_align1_batch: the regions "
                            "mem_align1_core returns)",
        "gpu_mem_align1_read_pairs_per_s": round(n_pairs / full_s, 1),
        "gpu_mem_align1_ms_per_batch": round(full_s * 1e3, 3),
        "cpu_oracle_mem_align1_read_pairs_per_s": round(n_pairs / (cpu_s + cpu_dedup_s), 1),
        "dedup_regions": int(droff[-1]),
        "dedup_regions_bit_exact_vs_oracle": dexact,
    }


def learned_schedule(ctx, L, param, d_jobs, n, d_seq, seq_bytes, d_out, cells_eval, jobs_eval, steps):
    """Plain-bound vs learned cost keys for the same jobs: model quality and makespan."""
    import torch
    from bsbolt_gb300 import _lib, cost_model as cm, extend, synth
    import ctypes
    t0 = time.perf_counter()
    tr_jobs, tr_seq = cached_jobs(1_000_000, 20261203 + 77)
    mat = synth.fill_scmat(1, 4)
    _, tr_cells = extend.ksw_extend2_batch(ctx, tr_jobs, tr_seq, mat, 6, 1, 6, 1, 100, want_cells=True)
    model = cm.CostModel(ctx, seed=11)
    dj = torch.from_numpy(tr_jobs.view(np.uint8).reshape(-1).copy()).cuda()
    ds = torch.from_numpy(tr_seq).cuda()
    feat = model.features(dj, len(tr_jobs), ds, len(tr_seq))
    losses = model.train(feat, torch.from_numpy(np.log1p(tr_cells).astype(np.float32)).cuda(), epochs=6)
    train_s = time.perf_counter() - t0
    del dj, ds, feat
    # inference on the benchmark jobs (timed on the device)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record()
    feat = model.features(d_jobs, n, d_seq, seq_bytes)
    pred, key = model.forward(feat, want_key=True)
    ev1.record()
    torch.cuda.synchronize()
    infer_ms = ev0.elapsed_time(ev1)
    pred_np = pred.cpu().numpy()
    bound = synth.cells_upper_bound(jobs_eval).astype(np.float64)

    jsz = synth.JOB_DTYPE.itemsize           # bsb_ext_job_t is 40 bytes

    def run(keyp, lo=0, hi=n):
        jb = ctypes.c_void_p(d_jobs.data_ptr() + lo * jsz)
        rc = L.bsb_extend_batch_device(ctx.handle, ctypes.byref(param), jb, hi - lo, ctypes.c_void_p(d_seq.data_ptr()),
                                       seq_bytes, ctypes.c_void_p(keyp + lo * 4) if keyp else None,
                                       ctypes.c_void_p(d_out.data_ptr() + lo * 24), None)
        _lib.check(ctx.handle, rc)

    def timed(keyp, chunk):
        s = torch.cuda.ExternalStream(ctx.stream)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(2):
            for lo in range(0, n, chunk):
                run(keyp, lo, min(n, lo + chunk))
        L.bsb_sync(ctx.handle)
        torch.cuda.synchronize()
        a.record(s)
        for _ in range(steps):
            for lo in range(0, n, chunk):
                run(keyp, lo, min(n, lo + chunk))
        b.record(s)
        torch.cuda.synchronize()
        _lib.check(ctx.handle, L.bsb_sync(ctx.handle))     # no job may have been skipped
        return a.elapsed_time(b) / steps

    kp = key.data_ptr()
    total_cells = float(cells_eval.sum())
    ref_out = d_out.cpu().numpy().copy()
    out = {}
    for label, chunk in (("whole_batch", n), ("batches_of_65536", 65536)):
        t_plain = timed(0, chunk)
        t_learn = timed(kp, chunk)
        same = bool(np.array_equal(d_out.cpu().numpy(), ref_out))
        out[label] = {"plain_ms": round(t_plain, 3), "learned_ms": round(t_learn, 3), "tuples_identical": same,
                      "plain_gcups": round(total_cells / t_plain / 1e6, 2),
                      "learned_gcups": round(total_cells / t_learn / 1e6, 2),
                      "speedup_learned_vs_plain": round(t_plain / t_learn, 4)}
    out.update({
        "model": "2x64 MLP, BF16 weights, FP32 accumulation, Adam, hand-written kernels (csrc/cost_mlp.cu)",
        "trained_on": "1M jobs of another seed, target log1p(cells logged by the extension kernel)",
        "train_s": round(train_s, 2), "train_loss_per_epoch": [round(x, 4) for x in losses],
        "inference_ms_4M_jobs": round(infer_ms, 3),
        "spearman_model": round(cm.spearman(pred_np, cells_eval), 4),
        "spearman_plain_bound": round(cm.spearman(bound, cells_eval), 4),
        "mape_model": round(cm.mape(np.expm1(pred_np), cells_eval), 4),
        "mape_plain_bound_calibrated": round(cm.mape(cm.calibrated_bound(bound, cells_eval), cells_eval), 4),
    })
    return out


def autotune_block(ctx, L, param, d_jobs, n, d_seq, seq_bytes, d_out, out_ref, steps):
    """Tile-shape autotuner: tune on a held-out job set of the same distribution, then time
    the headline batch with the tuned map against the default map (same device entry)."""
    import ctypes
    import torch
    from bsbolt_gb300 import _lib, autotune
    tj, ts = cached_jobs(1_000_000, 20261203 + 99)
    t0 = time.perf_counter()
    tmap, report = autotune.tune(ctx, tj, ts, param, min_jobs=4096, max_jobs=100_000, reps=2)
    tune_s = time.perf_counter() - t0

    def run(k):
        ms = []
        for _ in range(k + 1):
            rc = L.bsb_extend_batch_device(ctx.handle, ctypes.byref(param), ctypes.c_void_p(d_jobs.data_ptr()), n,
                                           ctypes.c_void_p(d_seq.data_ptr()), seq_bytes, None,
                                           ctypes.c_void_p(d_out.data_ptr()), None)
            _lib.check(ctx.handle, rc)
            _lib.check(ctx.handle, L.bsb_sync(ctx.handle))
            ms.append(ctx.last_kernel_ms())
        return float(np.median(ms[1:]))

    default_ms = run(steps)
    try:
        autotune.set_map(ctx, tmap)
        tuned_ms = run(steps)
        same = bool(np.array_equal(d_out.cpu().numpy(), out_ref))
    finally:
        autotune.set_map(ctx, None)
    changed = [r for r in report if r["best"] != r["current"]]
    return {"tuned_on": "1M held-out jobs of the same distribution (another seed), bands of need = qlen+1",
            "tune_s": round(tune_s, 2), "bands_tuned": len(report), "bands_changed": len(changed),
            "changes": [{"need": r["need"], "from": r["current"], "to": r["best"],
                         "ms": [r["current_ms"], r["best_ms"]]} for r in changed],
            "default_map_ms": round(default_ms, 3), "tuned_map_ms": round(tuned_ms, 3),
            "speedup_tuned_vs_default": round(default_ms / tuned_ms, 4), "tuples_identical": same}


def run_reference(args, ws, rank):
    from bsbolt_gb300 import synth
    if rank != 0:
        return
    jobs, seq = cached_jobs(args.jobs, rank_seed(0))
    mat = synth.fill_scmat(1, 4)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_reference_gcups(jobs, seq, args.ref_sample, threads, mat)
    vals, tms = [], []
    for _ in range(args.steps):
        g, dt, _, _, kind = cpu_reference_gcups(jobs, seq, args.ref_sample, threads, mat)
        vals.append(g)
        tms.append(dt)
    v = float(np.mean(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * float(np.mean(tms)), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded PCG64): the 4M-job extension workload's shapes",
        "config": {"workload": "batched ksw_extend2, 4M jobs, qlen U[10,140], w=100, BWA default scoring",
                   "sample_jobs_per_step": args.ref_sample, "parallelism": "host threads"},
        "cpu_baseline": {"value": round(v, 4), "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": f"first {args.ref_sample} of the 4M jobs per step, " +
                                   ("the reference's own ksw_extend2 (ksw.c:380-479 compiled from BSBolt's "
                                    "sources, oracle/_ref/libref_ksw.so)" if kind == "reference" else
                                    "ksw.c:380-479 CPU port (oracle/bsb_oracle.c)") +
                                   ", pthreads over all host cores"},
        "e2e": {"value": round(v, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, ws, rank, local):
    import torch

    from bsbolt_gb300 import _lib, extend, synth
    import ctypes

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    jobs, seq = cached_jobs(args.jobs, rank_seed(rank))
    n = len(jobs)
    mat = synth.fill_scmat(1, 4)
    ctx = extend.Context(local)
    L = ctx.L
    param = extend.make_param(mat, 6, 1, 6, 1, 100)

    # device-resident copies
    jobs_u8 = jobs.view(np.uint8).reshape(-1)
    d_jobs = torch.from_numpy(jobs_u8.copy()).to(f"cuda:{local}")
    d_seq = torch.from_numpy(seq).to(f"cuda:{local}")
    d_out = torch.zeros((n, 6), dtype=torch.int32, device=f"cuda:{local}")
    d_cells = torch.zeros(n, dtype=torch.int64, device=f"cuda:{local}")
    torch.cuda.synchronize()

    from bsbolt_gb300 import autotune
    shape_list = autotune.shapes(L)
    tmap = autotune.get_map(ctx)
    mapped = sorted(set(int(t) for t in tmap[1:]))          # shapes the device entry launches
    job_tile = tmap[jobs["qlen"].astype(np.int64) + 1]

    def step(with_cells=False):
        rc = L.bsb_extend_batch_device(ctx.handle, ctypes.byref(param), ctypes.c_void_p(d_jobs.data_ptr()), n,
                                       ctypes.c_void_p(d_seq.data_ptr()), len(seq), None,
                                       ctypes.c_void_p(d_out.data_ptr()),
                                       ctypes.c_void_p(d_cells.data_ptr()) if with_cells else None)
        _lib.check(ctx.handle, rc)

    # measured integer peaks (32-bit cells; 16-bit cells two per register)
    tops = ctypes.c_double()
    _lib.check(ctx.handle, L.bsb_probe_int_peak(ctx.handle, ctypes.byref(tops), None))
    int_peak = tops.value
    _lib.check(ctx.handle, L.bsb_probe_int16x2_peak(ctx.handle, ctypes.byref(tops), None))
    int16_peak = tops.value

    # reference cell count of this batch (the kernel's per-job count equals the
    # reference loop's, which the parity tests pin), and a parity sample
    step(with_cells=True)
    _lib.check(ctx.handle, L.bsb_sync(ctx.handle))
    total_cells = int(d_cells.sum().item())
    out_host = d_out.cpu().numpy()

    for _ in range(args.warmup):
        step()
    _lib.check(ctx.handle, L.bsb_sync(ctx.handle))

    s = torch.cuda.ExternalStream(ctx.stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kms = []
    tile_ms = np.zeros(_lib.BSB_NUM_TILES)
    tbuf = (ctypes.c_float * _lib.BSB_NUM_TILES)()
    with ClockSampler(local) as clk:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        ev0.record(s)
        for _ in range(args.steps):
            step()
            L.bsb_sync(ctx.handle)
            kms.append(ctx.last_kernel_ms())
            L.bsb_last_tile_ms(ctx.handle, tbuf, _lib.BSB_NUM_TILES)
            tile_ms += np.frombuffer(tbuf, dtype=np.float32)
        ev1.record(s)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    clocks = clk.summary()
    elapsed_ms = ev0.elapsed_time(ev1)
    elapsed_ms, all_cells = replica_totals(elapsed_ms, total_cells, dist, f"cuda:{local}")
    ms_step = elapsed_ms / args.steps
    value = all_cells / (ms_step * 1e-3) / 1e9
    kernel_ms = float(np.mean(kms))
    achieved_all = total_cells * INT_OPS_PER_CELL / (kernel_ms * 1e-3) / 1e12
    # the dominant kernel: the tile shape with the most device time per step (CUDA events
    # on the context stream around each shape's launch), and the cells its jobs hold
    tile_ms /= args.steps
    cells_host = d_cells.cpu().numpy()
    tile_cells = np.bincount(job_tile, weights=cells_host.astype(np.float64), minlength=_lib.BSB_NUM_TILES)
    tile_jobs = np.bincount(job_tile, minlength=_lib.BSB_NUM_TILES)
    dom = int(np.argmax(tile_ms))
    dom_ms = float(tile_ms[dom])
    achieved = tile_cells[dom] * INT_OPS_PER_CELL / (dom_ms * 1e-3) / 1e12
    dom_g, dom_c = shape_list[dom]
    dom16 = dom_c % 2 == 0 and dom_c <= 32    # even C up to 32: 16-bit cells (the jobs of this batch all fit)
    dom_name = ("ksw_tile16_kernel<%d,%d>" % (dom_c // 2, dom_g)) if dom16 else ("ksw_tile_kernel<%d,%d>" % (dom_c, dom_g))
    dom_peak = int16_peak if dom16 else int_peak
    cells16_frac = float(sum(tile_cells[t] for t in range(len(shape_list))
                             if shape_list[t][1] % 2 == 0 and shape_list[t][1] <= 32)
                         / max(tile_cells.sum(), 1.0))
    traffic = None
    prof = os.path.join(ROOT, "profiles", "ksw_tile_kernel_traffic.txt")
    if os.path.exists(prof):       # DRAM bytes per job of this shape from an ncu capture
        for ln in open(prof):
            f = ln.split()
            if len(f) >= 3 and f[0] == "%dx%d" % shape_list[dom] and f[1] == "dram_bytes_per_job":
                traffic = int(float(f[2]) * tile_jobs[dom])

    # end to end through the C ABI with pinned host buffers
    hj = torch.from_numpy(jobs_u8).pin_memory()
    hs = torch.from_numpy(seq).pin_memory()
    ho = torch.zeros((n, 6), dtype=torch.int32).pin_memory()
    def e2e_step():
        rc = L.bsb_extend_batch(ctx.handle, ctypes.byref(param), ctypes.c_void_p(hj.data_ptr()), n,
                                ctypes.c_void_p(hs.data_ptr()), len(seq), ctypes.c_void_p(ho.data_ptr()), None)
        _lib.check(ctx.handle, rc)
    e2e_step()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 5))
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_s, _ = replica_totals(e2e_s, 0, dist, f"cuda:{local}")
    e2e_val = all_cells / e2e_s / 1e9
    e2e_match = bool(np.array_equal(ho.numpy(), out_host))

    cpu = None
    parity = None
    if rank == 0:
        threads = os.cpu_count() or 1
        g, dt, ref_out, ref_cells, kind = cpu_reference_gcups(jobs, seq, args.cpu_sample, threads, mat)
        parity = bool(np.array_equal(ref_out, out_host[: args.cpu_sample]))
        cells_match = int(ref_cells.sum()) == int(d_cells[: args.cpu_sample].sum().item())
        cpu = {"value": round(g, 4), "unit": UNIT, "cores": threads, "kind": kind,
               "sample": f"first {args.cpu_sample} jobs ({int(ref_cells.sum())} cells, {dt:.2f} s wall), " +
                         ("the reference's own ksw_extend2 compiled from BSBolt's sources" if kind == "reference"
                          else "CPU port of ksw.c:380-479") + ", pthreads over all host cores",
               "tuples_bit_exact_on_sample": parity, "cells_match_on_sample": bool(cells_match)}

    learned = None
    if rank == 0 and not args.no_learned:
        try:
            learned = learned_schedule(ctx, L, param, d_jobs, n, d_seq, len(seq), d_out,
                                       d_cells.cpu().numpy(), jobs, max(3, min(args.steps, 5)))
        except Exception as e:   # reported, never hidden
            learned = {"error": f"{type(e).__name__}: {e}"}

    big = rrbs = None
    if rank == 0 and not args.no_ref100mb:
        try:
            big = pipeline_ref100mb(ctx)
        except Exception as e:   # reported, never hidden
            big = {"error": f"{type(e).__name__}: {e}"}
        try:
            rrbs = pipeline_rrbs(ctx)
        except Exception as e:   # reported, never hidden
            rrbs = {"error": f"{type(e).__name__}: {e}"}

    big1g = big3g = None
    if rank == 0 and args.ref1gb:
        try:
            big1g = pipeline_ref1gb(ctx, n_pairs=args.ref1gb_pairs)
        except Exception as e:   # reported, never hidden
            big1g = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0 and not args.no_ref3gb:
        try:
            big3g = pipeline_ref1gb(ctx, n_pairs=args.ref3gb_pairs, tag="3gb", learned=not args.no_learned)
        except Exception as e:   # reported, never hidden
            big3g = {"error": f"{type(e).__name__}: {e}"}

    lp = None
    if rank == 0 and not args.no_learned and not args.no_ref100mb:
        try:
            lp = learned_pipeline(ctx)
        except Exception as e:   # reported, never hidden
            lp = {"error": f"{type(e).__name__}: {e}"}

    tuned = None
    if rank == 0 and not args.no_autotune:
        try:
            tuned = autotune_block(ctx, L, param, d_jobs, n, d_seq, len(seq), d_out, out_host,
                                   max(3, min(args.steps, 5)))
        except Exception as e:   # reported, never hidden
            tuned = {"error": f"{type(e).__name__}: {e}"}

    secondary = None
    if rank == 0 and not args.no_pipeline:
        try:
            secondary = pipeline_secondary(ctx, args.steps, rank)
        except Exception as e:   # reported, never hidden
            secondary = {"error": f"{type(e).__name__}: {e}"}

    cig = None
    if rank == 0 and not args.no_cigar:
        try:
            cig = cigar_block(ctx, args.steps)
        except Exception as e:   # reported, never hidden
            cig = {"error": f"{type(e).__name__}: {e}"}

    msw = None
    if rank == 0 and not args.no_matesw:
        try:
            msw = matesw_block(ctx, args.steps)
        except Exception as e:   # reported, never hidden
            msw = {"error": f"{type(e).__name__}: {e}"}

    sam = None
    if rank == 0 and not args.no_sam:
        try:
            sam = sam_block(0 if args.no_ref100mb else args.sam_pairs, 0 if args.no_ref100mb else args.sam_rrbs)
        except Exception as e:   # reported, never hidden
            sam = {"error": f"{type(e).__name__}: {e}"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int16x2" if cells16_frac >= 0.5 else "int32",
            "data": "synthetic (seeded PCG64): the 4M-job extension workload's shapes",
            "config": {"workload": "batched ksw_extend2, 4M jobs, qlen U[10,140], target=query+100nt "
                                   "(1% sub, 0.1% indel, 20% unrelated), h0 U[19,100], w=100, a1 b4 o6 e1 z100 L5",
                       "jobs": n, "cells_per_step": total_cells, "seq_bytes": int(len(seq)),
                       "l2": "inputs 1.0 GB > 129 MB L2 per step (no flush needed)",
                       "schedule": "plain (default tile map, longest bound first)", "parallelism": f"replicas x{ws}"},
            "roofline": {"bound": "int", "achieved": round(achieved, 3), "peak": round(dom_peak, 3),
                         "unit": "Tops/s", "frac": round(achieved / dom_peak, 4), "traffic": traffic,
                         "kernel": dom_name, "kernel_ms_per_launch": round(dom_ms, 4),
                         "kernel_cells_per_launch": int(tile_cells[dom]),
                         "kernel_share_of_step": round(dom_ms / kernel_ms, 4),
                         "peak_source": ("measured add+max throughput on 16-bit pairs (__viaddmax_s16x2, "
                                         "bsb_probe_int16x2_peak) on this GPU, the width this kernel computes in"
                                         if dom16 else
                                         "measured add+max int32 throughput (bsb_probe_int_peak) on this GPU") +
                                        "; MEASURED_PEAKS.json has no integer figure",
                         "int32_peak": round(int_peak, 3), "int16x2_peak": round(int16_peak, 3),
                         "ops_per_cell": INT_OPS_PER_CELL,
                         "all_kernels": {"achieved": round(achieved_all, 3),
                                         "frac": round(achieved_all / (int16_peak if cells16_frac >= 0.5 else int_peak), 4),
                                         "cells_on_16bit_kernels": round(cells16_frac, 4),
                                         "ms_per_step": round(kernel_ms, 4)}},
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_val, 3), "unit": UNIT,
                    "h2d_bytes_per_step": int(jobs_u8.nbytes + len(seq)), "d2h_bytes_per_step": int(n * 24),
                    "tuples_match_device_run": e2e_match, "s_per_step": round(e2e_s, 4)},
            "gpu_launches": (SCHED_KERNELS + sum(2 if shape_list[t][1] % 2 == 0 and shape_list[t][1] <= 32 else 1
                                                 for t in mapped)) * args.steps,
            "clocks": clocks,
            "pipeline": secondary,
            "learned_schedule": learned,
            "learned_read_order_rrbs": lp,
            "autotune": tuned,
            "pipeline_100mb_ref": big,
            "pipeline_rrbs_100mb_ref": rrbs,
            "gen_cigar": cig,
            "mate_rescue_sw": msw,
            "sam_pipeline": sam,
            "pipeline_1gb_ref": big1g,
            "pipeline_3gb_ref": big3g,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--jobs", type=int, default=4_000_000)
    ap.add_argument("--cpu-sample", type=int, default=1_000_000)
    ap.add_argument("--ref-sample", type=int, default=200_000)
    ap.add_argument("--no-pipeline", action="store_true", help="skip the seeds->regions secondary block")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-schedule block")
    ap.add_argument("--no-autotune", action="store_true", help="skip the tile-shape autotuner block")
    ap.add_argument("--no-cigar", action="store_true", help="skip the bwa_gen_cigar2 block")
    ap.add_argument("--no-matesw", action="store_true", help="skip the mate-rescue Smith-Waterman block")
    ap.add_argument("--no-ref100mb", action="store_true",
                    help="skip the 100 Mb-reference blocks, WGBS-like PE and RRBS-like SE (they build a 100 Mb "
                         "index: ~1 min the first time)")
    ap.add_argument("--no-sam", action="store_true", help="skip the stock bwa vs bwa_gpu SAM block")
    ap.add_argument("--ref1gb", action="store_true",
                    help="add the 1 Gb-reference block (index sorted on the GPU; a few minutes to build)")
    ap.add_argument("--ref1gb-pairs", type=int, default=200_000)
    ap.add_argument("--no-ref3gb", action="store_true",
                    help="skip the 3.1 Gb human-scale block (24 contigs, 45%% repeats; the index is sorted on "
                         "the GPU with 64-bit ranks: ~3 min and ~200 GB of device memory the first time)")
    ap.add_argument("--ref3gb-pairs", type=int, default=200_000)
    ap.add_argument("--sam-pairs", type=int, default=500_000,
                    help="2x150 pairs of the SAM block on the 100 Mb reference (the full workload is 4M)")
    ap.add_argument("--sam-rrbs", type=int, default=1_000_000,
                    help="RRBS-like reads of the SAM block (the full workload is 3M)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
