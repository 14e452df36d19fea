"""The multi-process path on CPU (two gloo ranks): replicas only.

The seed-extend path shards by batch with no exchange step, so N processes run N
independent batches.  What the N > 1 run adds is host-side: each rank draws its own
workload, the whole-job time is the slowest rank's and the work is every rank's
(bench.replica_totals), and under torchrun the reference arm prints one line from
rank 0 while the other ranks exit 0 without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    elapsed = [12.5, 20.0][rank]
    cells = [1000, 3000][rank]
    t, c = bench.replica_totals(elapsed, cells, dist, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t, c, bench.rank_seed(rank)))


def test_replica_totals_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, c, seed in res:
        assert t == 20.0 and c == 4000.0          # slowest rank's time, every rank's cells
    assert res[0][3] != res[1][3]                 # each replica extends its own batch


def test_replica_totals_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_totals(7.0, 42) == (7.0, 42.0)


def test_reference_arm_under_torchrun_prints_one_line(tmp_path):
    """`bench.py --impl reference` launched as two ranks: rank 0 times the CPU
    implementation and prints the line; rank 1 exits 0 without work."""
    pytest.importorskip("torch")
    port = free_port()
    env = dict(os.environ, TMPDIR=str(tmp_path))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--jobs", "4000",
           "--ref-sample", "2000"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    import oracle
    kind = "reference" if oracle.have_reference_ksw() else "port"     # the compiled reference where it was built
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == kind
