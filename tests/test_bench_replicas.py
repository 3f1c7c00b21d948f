"""The multi-GPU path of bench.py on the CPU: replicas (one per rank, no data-path
collective) whose whole-job rate uses the slowest rank's time, reduced over a world-size-2
`gloo` group; and the reference arm, which only rank 0 runs."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, times, q):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        t = bench.max_over_ranks(times[rank], dist, "cpu")
        q.put((rank, t, bench.job_rate(ws, 1 << 22, 20, t)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_rate_uses_slowest_rank():
    import torch.multiprocessing as mp

    ws, times = 2, [1.25, 2.5]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, ws, port, times, q)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(ws))
    for rank, t, rate in got:
        assert t == max(times)
        assert rate == ws * (1 << 22) * 20 / max(times)


def test_single_rank_helpers():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(3.0) == 3.0
    assert bench.job_rate(1, 100, 2, 4.0) == 50.0


def test_reference_arm_only_on_rank0():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2"], env=env,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
