"""`bsbolt Align` on the GPU: the same options, the same `bwa mem` command line, the same
mapping statistics, with `bwa_gpu` (BSBolt's BWA fork linked to libbsbgpu.so) as the aligner.

    python -m bsbolt_gb300.align -DB <db> -F1 r1.fq [-F2 r2.fq] -O out [-t 16] [...]

Mirrors bsbolt/Utils/Launcher.py:75-115 (`launch_alignment`: the argv built from the
parsed options, bsbolt/Utils/Parser.py:31-115 for their defaults) and
bsbolt/Align/AlignReads.py:43-87 (`BisulfiteAlignmentAndProcessing.align_reads`: stderr
watched for `BSStat <category>: <count>` lines, summed into the mapping statistics).
One difference: the reference pipes SAM into htslib's stream_bam to write `<O>.bam`;
BAM compression is not part of this path, so the SAM is written to `<O>.sam` (or stdout
with -OS).
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BWA_GPU = os.path.join(HERE, "integration", "_build", "bwa_gpu")

# the options of `bsbolt Align` that reach `bwa mem`, with bsbolt's defaults (Parser.py:31-115)
DEFAULTS = dict(UN=False, CP=0.5, CT=5, SP=0.1, t=1, k=19, w=100, d=100, r=1.5, y=20, c=500, D=0.50, W=0,
                m=50, S=False, A=1, B=4, INDEL="6,6", E="1,1", L="30,30", U=17, p=False, H=None, j=False,
                T=10, XA="100,200", DR=0.95, M=False, I=None)


def bwa_command(bwa: str, db: str, f1: str, f2: str | None = None, **opts) -> list:
    """The `bwa mem` argv `bsbolt Align` builds (Launcher.py:75-103), for the binary `bwa`."""
    o = dict(DEFAULTS)
    unknown = set(opts) - set(o)
    if unknown:
        raise TypeError(f"unknown Align options: {sorted(unknown)}")
    o.update(opts)
    cmd = [bwa, "mem", "-Y"]
    if o["UN"]:
        cmd.append("-z")
    for a in ("M", "S", "j", "p"):
        if o[a]:
            cmd.append(f"-{a}")
    for a in ("A", "B", "D", "E", "L", "T", "U", "W", "c", "d", "k", "m", "r", "t", "w", "y"):
        cmd += [f"-{a}", str(o[a])]
    if o["H"] is not None:
        cmd += ["-H", str(o["H"])]
    if o["I"] is not None:
        cmd += ["-I", str(o["I"])]
    if o["INDEL"]:
        cmd += ["-O", str(o["INDEL"])]
    if o["XA"]:
        cmd += ["-h", str(o["XA"])]
    cmd += ["-e", str(o["SP"]), "-l", str(o["CP"]), "-n", str(o["CT"]), "-Z", str(o["DR"])]
    if not db.endswith(".fa"):
        db = os.path.join(db, "BSB_ref.fa")
    cmd.append(db)
    cmd.append(f1)
    if f2 is not None:
        cmd.append(f2)
    return cmd


def mapping_statistics() -> dict:
    return dict(TotalReads=0, TotalAlignments=0, BSAmbiguous=0, C_C2T=0, C_G2A=0, W_C2T=0, W_G2A=0, Unaligned=0)


def run_alignment(cmd: list, sam_out, extra_args: list | None = None, env=None, echo=True,
                  keep: list | None = None) -> dict:
    """Runs `cmd` (+ extra_args, e.g. ["-K", "10000000"] after `mem`), SAM to the open binary
    file sam_out, and returns the summed `BSStat` counts of its stderr (AlignReads.py:60-70).
    Other stderr lines are echoed (echo) and/or appended to `keep`.  Raises RuntimeError when
    the aligner fails, as the reference raises BisulfiteAlignmentError."""
    if extra_args:
        cmd = cmd[:2] + list(extra_args) + cmd[2:]
    stats = mapping_statistics()
    proc = subprocess.Popen(cmd, stdout=sam_out, stderr=subprocess.PIPE, universal_newlines=True, env=env)
    for line in proc.stderr:
        if line.startswith("BSStat "):
            category, count = line[7:].split(": ")
            stats[category] += int(count)
            if echo:
                print(line[7:].strip(), file=sys.stderr)
        else:
            if echo:
                print(line.rstrip("\n"), file=sys.stderr)
            if keep is not None:
                keep.append(line.rstrip("\n"))
    if proc.wait():
        raise RuntimeError(f"alignment failed with exit code {proc.returncode}: {' '.join(cmd)}")
    return stats


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="bsbolt_gb300.align", description=__doc__.split("\n")[0])
    ap.add_argument("-F1", required=True)
    ap.add_argument("-F2", default=None)
    ap.add_argument("-DB", required=True)
    ap.add_argument("-O", default=None)
    ap.add_argument("-OS", action="store_true")
    ap.add_argument("-BWA", default=BWA_GPU, help="aligner binary (default: bwa_gpu of this package)")
    for k, v in DEFAULTS.items():
        if isinstance(v, bool):
            ap.add_argument(f"-{k}", action="store_true", default=v)
        else:
            ap.add_argument(f"-{k}", type=type(v) if v is not None else str, default=v)
    a = ap.parse_args(argv)
    if a.O is None and not a.OS:
        ap.error("-O and -OS arguments empty, please specify output path")
    opts = {k: getattr(a, k) for k in DEFAULTS}
    cmd = bwa_command(a.BWA, a.DB, a.F1, a.F2, **opts)
    print(" ".join(cmd), file=sys.stderr)
    if a.OS:
        stats = run_alignment(cmd, sys.stdout.buffer)
    else:
        with open(f"{a.O}.sam", "wb") as f:
            stats = run_alignment(cmd, f)
    for k, v in stats.items():
        print(f"{k}: {v}", file=sys.stderr)
    return 0


if __name__ == "__main__":
    sys.exit(main())
