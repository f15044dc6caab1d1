"""The multi-GPU contract of bench.py, on CPU ranks (gloo, world size 2).

Every group of V matrices is independent, so N GPUs run N replicas with no
collective on the data path; the only cross-rank step is the timing
reduction (the slowest rank decides the whole-job throughput). That step is
tested here with two gloo ranks that report different times, and the
reference arm is launched through torchrun with two ranks: rank 0 alone
prints the one JSON line and the other rank exits 0 without work.
"""
import json
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        times = [10.0 + 5.0 * rank, 20.0 - 5.0 * rank]   # each rank slowest once
        out[rank] = (bench.slowest_rank(times, "cpu"),
                     bench.job_throughput(1000, bench.slowest_rank([4.0 * (rank + 1)], "cpu")[0],
                                          ws))
    finally:
        dist.destroy_process_group()


def test_slowest_rank_decides_on_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(2):
            times, value = out[r]
            assert times == [15.0, 20.0]                 # max over ranks, per entry
            assert value == 2 * 1000 / (8.0 * 1e-3)      # all units over the slowest time


def test_single_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.slowest_rank([3.0, 4.0]) == [3.0, 4.0]
    assert bench.job_throughput(500, 2.0, 1) == 250000.0


def test_reference_arm_under_torchrun_prints_once(oracle_lib):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3",
           "--ref-per-n", "1024"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600,
                       env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["steps"] == 1
    assert line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
