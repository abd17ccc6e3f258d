"""CPU, two gloo ranks: the benchmark's multi-rank bookkeeping.  Every rank
renders its own views (replicas; the path has no exchange step), the job's
time is the slowest rank's, and the whole-job rate counts every rank's
frames.  The reference arm runs on rank 0 alone."""
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took 10*(r+1) ms for its frames and 20*(r+1) end to end
        t, e = bench.max_over_ranks([10.0 * (rank + 1), 20.0 * (rank + 1)], "cpu")
        q.put((rank, t, e, bench.whole_job_rate(5, world, t)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, t, e, rate in got:
        assert t == 20.0 and e == 40.0          # the slowest rank's times on every rank
        assert rate == pytest.approx(5 * 2 / 0.020)  # all ranks' frames over that time


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([1.5, 2.5], "cpu") == [1.5, 2.5]
    assert bench.whole_job_rate(10, 1, 500.0) == pytest.approx(20.0)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "plain_128", "--steps", "1", "--warmup", "1"], env=env, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_reference_arm_line():
    """The reference arm's JSON line: the CPU restatement timed on the host's
    cores, with the contract's keys."""
    import json
    env = dict(os.environ, RANK="0", WORLD_SIZE="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "plain_128", "--steps", "2", "--warmup", "1"], env=env, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "frames/s"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert "layout" not in line["config"]


def test_reference_arm_learned_line_has_our_config():
    """The reference arm on the learned-skip workload (the small variant):
    the oracle on bands of the same frames, and the same config dict as the
    GPU arm's line, so that the two lines describe one workload."""
    import argparse
    import json
    import bench
    env = dict(os.environ, RANK="0", WORLD_SIZE="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "learned_256", "--steps", "2", "--warmup", "1"], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["dtype"] == "u16"
    args = argparse.Namespace(gpus=1)
    assert line["config"] == bench.learned_config(args, bench.LEARNED_SMALL)
