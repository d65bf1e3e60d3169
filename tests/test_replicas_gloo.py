"""Multi-GPU is replicas only (pixels and samples are independent): N ranks
render interleaved samples and bench.py reports every rank's rays over the
slowest rank's time.  These tests run that host logic as two gloo ranks on the
CPU, and the reference arm under torchrun with two ranks (rank 0 alone
prints its line)."""
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    r, w, local = bench.dist_env()
    D = bench.Dist(w, local)
    D.barrier()
    # rank r traced (r + 1) million rays in 10 (r + 1) ms
    value, ms_max = bench.replica_throughput(D, 1e6 * (r + 1), 10.0 * (r + 1))
    D.barrier()
    D.close()
    q.put((r, value, ms_max))


def test_replica_throughput_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = sorted(q.get(timeout=120) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=30)
            if p.is_alive():
                p.kill()
    assert [g[0] for g in got] == [0, 1]
    for _, value, ms_max in got:
        assert ms_max == 20.0
        assert value == pytest.approx(3e6 / 0.020 / 1e6)  # 3M rays over the slowest rank's 20 ms


def test_reference_arm_two_ranks_rank0_prints():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "3", "--subdivisions", "3", "--width", "64", "--height", "32",
           "--cpu-seconds", "0.5"]
    out = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
