"""The N>1 path of bench.py on CPU: world_size-2 gloo ranks (one process each, rendezvous on
127.0.0.1) agree on the max-over-ranks duration and on the whole-job rate, and the reference arm's
non-zero ranks exit without work or output."""
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 10.0 + 5.0 * rank  # the slower rank sets the job's duration
        m = bench.max_over_ranks(ms, dist, "cpu")
        rate = bench.whole_job_rate(1000, 4, world, m)
        dist.barrier()
        out[rank] = (m, rate)
    finally:
        dist.destroy_process_group()


def test_bench_ranks_agree_on_max_and_rate():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_rank, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
        res = dict(out)
    assert sorted(res) == [0, 1]
    for m, rate in res.values():
        assert m == 15.0
        assert rate == pytest.approx(2 * 1000 * 4 / 15e-3)


def test_reference_arm_nonzero_rank_exits_quietly():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
