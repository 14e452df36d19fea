"""In-tree build of the sm_103a library (libbsbgpu.so) and the host index builder.

    python -m bsbolt_gb300.build          # or __graft_entry__.build()

Each CUDA translation unit is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo``, then linked
into ``bsbolt_gb300/lib/libbsbgpu.so`` with the CUDA runtime linked
statically, so the library needs no torch and no extra shared objects.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(HERE, "_build")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = GENCODE + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                        "--expt-relaxed-constexpr"]

LIB_GPU = os.path.join(LIBDIR, "libbsbgpu.so")
LIB_HOST = os.path.join(LIBDIR, "libbsbhost.so")


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the sm_103a library cannot be built")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
            + glob.glob(os.path.join(HERE, "..", "include", "*.h")))


def build(force: bool = False, verbose: bool = False) -> None:
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    cus = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    objs = []
    jobs = []
    for cu in cus:
        obj = os.path.join(OBJDIR, os.path.basename(cu)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [cu] + hdrs):
            cmd = [nvcc] + NVCC_FLAGS + ["-c", cu, "-o", obj]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(subprocess.run, cmd, capture_output=True, text=True) for cmd in jobs]
            for cmd, f in zip(jobs, futs):
                r = f.result()
                if verbose or r.returncode != 0:
                    print(" ".join(cmd))
                    print(r.stdout, r.stderr)
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed for %s" % cmd[-3])
    if force or jobs or _stale(LIB_GPU, objs):
        tmp = LIB_GPU + ".tmp%d" % os.getpid()
        subprocess.check_call([nvcc] + GENCODE + ["-shared", "-cudart", "static", "-o", tmp] + objs)
        os.replace(tmp, LIB_GPU)
    # host-only C: index builder (SA-IS + BWA on-disk formats)
    host_src = sorted(glob.glob(os.path.join(CSRC, "host_*.c")))
    if host_src and (force or _stale(LIB_HOST, host_src + hdrs)):
        tmp = LIB_HOST + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-pthread", "-std=gnu11", "-o", tmp]
                              + host_src)
        os.replace(tmp, LIB_HOST)


if __name__ == "__main__":
    build(verbose=True)
