"""The multi-process (replica) path of bench.py on CPU: two gloo ranks with
different local step times agree on the job's step time (the slowest rank)
and on the whole-job throughput; under torchrun the reference arm runs on
rank 0 only and the other ranks exit without work."""
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, out):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, REPO)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        local_ms = 10.0 + 5.0 * rank  # rank 1 is slower
        ms = bench.max_over_ranks(local_ms, ws, torch.device("cpu"))
        out.put((rank, ms, bench.job_value(2_000_000, ms, ws)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_step():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]
    assert res[0][2] == res[1][2] == pytest.approx(2 * 2_000_000 / 15e-3)


def test_single_rank_is_the_identity():
    sys.path.insert(0, REPO)
    import bench

    assert bench.max_over_ranks(3.5, 1, None) == 3.5
    assert bench.job_value(1000, 2.0, 1) == pytest.approx(5e5)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "0"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
