"""The multi-GPU path of bench.py is replicas only: each rank sweeps its own disjoint set of chains
and the ranks meet only in scalar reductions (max of the timed region, sums of the counts).  These
tests run that host logic as two gloo ranks on the CPU."""

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
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    r, w, local = bench.dist_setup(None)
    mx = bench.barrier_max(w, 10.0 + 5 * r)
    sm = bench.barrier_sum(w, r + 1)
    bench.barrier(w)
    q.put((r, w, local, mx, sm, list(bench.replica_streams(r, 3))))
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_and_shard():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, l0, mx0, sm0, s0), (r1, w1, l1, mx1, sm1, s1) = out
    assert (r0, r1) == (0, 1) and w0 == w1 == 2 and (l0, l1) == (0, 1)
    assert mx0 == mx1 == 15.0  # max over ranks of the timed region
    assert sm0 == sm1 == 3.0  # whole-job sums
    assert s0 == [0, 1, 2] and s1 == [3, 4, 5]  # disjoint chains


def test_reference_arm_prints_once_under_two_ranks():
    """--impl reference under torchrun: rank 0 runs the CPU path and prints one JSON line, the
    other rank exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--side", "4", "--beta", "1", "--cpu-sweeps", "4",
           "--cpu-threads", "2"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
