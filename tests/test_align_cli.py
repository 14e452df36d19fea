"""bsbolt_gb300.align mirrors `bsbolt Align`: the same `bwa mem` argv from the same options
(bsbolt/Utils/Launcher.py:75-103, defaults bsbolt/Utils/Parser.py:31-115) and the same mapping
statistics from the aligner's `BSStat` lines (bsbolt/Align/AlignReads.py:60-70).  CPU: the
argv and, with the stock `bwa` where the reference was built, the statistics."""
import os
import sys

import pytest

from bsbolt_gb300 import align

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BWA = os.path.join(ROOT, "oracle", "_ref", "bwa")
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import sam_sets  # noqa: E402


def test_default_argv_is_bsbolt_aligns():
    cmd = align.bwa_command("bwa", "db", "r1.fq", "r2.fq")
    assert cmd == ["bwa", "mem", "-Y", "-A", "1", "-B", "4", "-D", "0.5", "-E", "1,1", "-L", "30,30", "-T", "10",
                   "-U", "17", "-W", "0", "-c", "500", "-d", "100", "-k", "19", "-m", "50", "-r", "1.5", "-t", "1",
                   "-w", "100", "-y", "20", "-O", "6,6", "-h", "100,200", "-e", "0.1", "-l", "0.5", "-n", "5",
                   "-Z", "0.95", os.path.join("db", "BSB_ref.fa"), "r1.fq", "r2.fq"]
    # the test sets' argv is the same option list
    flat = cmd[3:-3]
    i = flat.index("-t")
    assert flat[:i] + flat[i + 2:] == sam_sets.BSBOLT_ARGS


def test_flags_and_options():
    cmd = align.bwa_command("bwa", "ref.fa", "r1.fq", UN=True, S=True, M=True, L="5,5", t=16, I="300,30", H="x")
    assert cmd[:6] == ["bwa", "mem", "-Y", "-z", "-M", "-S"]
    assert cmd[cmd.index("-L") + 1] == "5,5" and cmd[cmd.index("-t") + 1] == "16"
    assert cmd[cmd.index("-I") + 1] == "300,30" and cmd[cmd.index("-H") + 1] == "x"
    assert cmd[-2:] == ["ref.fa", "r1.fq"]
    with pytest.raises(TypeError):
        align.bwa_command("bwa", "ref.fa", "r1.fq", nonsense=1)


@pytest.mark.skipif(not os.path.exists(BWA), reason="reference bwa not built here")
def test_mapping_statistics_from_bsstat(tmp_path):
    fa, r1, r2 = sam_sets.pe_set(str(tmp_path), BWA)[:3]
    cmd = align.bwa_command(BWA, fa, r1, r2, t=4)
    with open(tmp_path / "out.sam", "wb") as f:
        st = align.run_alignment(cmd, f, echo=False)
    assert st["TotalReads"] == 3080          # bs_sorter counts a pair once
    assert st["W_C2T"] + st["C_C2T"] + st["W_G2A"] + st["C_G2A"] > 0.9 * st["TotalReads"]
    assert set(st) == set(align.mapping_statistics())
