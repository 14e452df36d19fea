"""The C ABI's record layouts (include/bsbgpu.h) equal their Python mirrors, field by field:
sizes and offsets from a small C program compiled against the header (CPU only)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from bsbolt_gb300 import _lib, cigar, matesw, seed, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# C struct -> (Python mirror, fields whose offsets are compared)
RECORDS = {
    "bsb_ext_param_t": (_lib.ExtParam, ["mat", "o_del", "e_del", "o_ins", "e_ins", "zdrop"]),
    "bsb_seed_opt_t": (_lib.SeedOpt, ["min_seed_len", "split_factor", "split_width", "max_mem_intv"]),
    "bsb_index_view_t": (_lib.IndexView, ["primary", "L2", "bwt", "bwt_size", "sa", "n_sa", "sa_intv", "pac",
                                          "l_pac", "n_seqs", "ann_offset", "ann_len"]),
    "bsb_align_opt_t": (_lib.AlignOpt, ["a", "b", "o_del", "e_del", "o_ins", "e_ins", "w", "zdrop", "pen_clip5",
                                        "pen_clip3", "min_seed_len", "max_occ", "max_chain_gap", "min_chain_weight",
                                        "max_chain_extend", "mask_level", "drop_ratio", "split_factor",
                                        "split_width", "max_mem_intv", "mat", "mask_level_redun"]),
    "bsb_ext_job_t": (synth.JOB_DTYPE, ["qoff", "toff", "qlen", "tlen", "h0", "w", "end_bonus", "flags"]),
    "bsb_reg_t": (seed.REG_DTYPE, ["rb", "re", "qb", "qe", "rid", "score", "truesc", "w", "seedcov", "seedlen0",
                                   "frac_rep", "n_comp"]),
    "bsb_cigar_job_t": (cigar.JOB_DTYPE, ["rb", "re", "qoff", "ooff", "l_query", "w"]),
    "bsb_cigar_out_t": (cigar.OUT_DTYPE, ["score", "n_cigar", "NM", "cg_meth", "cg_unmeth", "ch_meth", "ch_unmeth",
                                          "status", "off", "bytes"]),
    "bsb_sw_job_t": (matesw.JOB_DTYPE, ["qoff", "toff", "qlen", "tlen", "xtra"]),
    "bsb_kswr_t": (matesw.KSWR_DTYPE, ["score", "te", "qe", "score2", "te2", "tb", "qb"]),
}


def _fields(mirror):
    if isinstance(mirror, np.dtype):
        return mirror.itemsize, {f: mirror.fields[f][1] for f in mirror.names}
    return ctypes.sizeof(mirror), {f[0]: getattr(mirror, f[0]).offset for f in mirror._fields_}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "bsbgpu.h"', 'int main(void) {']
    for name, (mirror, fields) in RECORDS.items():
        lines.append(f'    printf("{name} size %zu\\n", sizeof({name}));')
        for f in fields or []:
            lines.append(f'    printf("{name} {f} %zu\\n", offsetof({name}, {f}));')
    lines += ['    return 0;', '}']
    d = tmp_path_factory.mktemp("abi")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = {}
    for ln in subprocess.check_output([str(exe)]).decode().splitlines():
        name, field, v = ln.split()
        out[(name, field)] = int(v)
    return out


@pytest.mark.parametrize("name", sorted(RECORDS))
def test_record_layout_matches_python(c_layout, name):
    mirror, fields = RECORDS[name]
    size, offsets = _fields(mirror)
    assert c_layout[(name, "size")] == size, f"{name}: C {c_layout[(name, 'size')]} bytes, Python {size}"
    for f in fields or []:
        assert c_layout[(name, f)] == offsets[f], f"{name}.{f}: C offset {c_layout[(name, f)]}, Python {offsets[f]}"
