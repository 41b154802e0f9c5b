"""The N > 1 benchmark path on CPU: world_size-2 gloo ranks exercise the
replica plumbing (barrier, max-over-ranks timing, whole-job rate) that
bench.py uses with NCCL on GPUs; and the reference arm's rank gating under
a torchrun-style environment."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    from amuse_gb300 import replicas
    assert replicas.env() == (rank, world, rank)
    assert replicas.init("gloo") == world
    replicas.barrier()
    seconds = 0.5 + rank          # rank 1 is the slow one
    slowest = replicas.max_over_ranks(seconds)
    rate = replicas.whole_job_rate(1000.0, world, slowest)
    replicas.finalize()
    q.put((rank, slowest, rate))


def test_two_gloo_ranks_max_over_ranks_and_whole_job_rate():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(world))
    for rank, slowest, rate in res:
        assert slowest == 1.5                       # both ranks see the slowest time
        assert rate == pytest.approx(2 * 1000.0 / 1.5)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    from amuse_gb300 import replicas
    env = {k: os.environ.pop(k) for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK") if k in os.environ}
    try:
        assert replicas.init("gloo") == 1
        assert replicas.max_over_ranks(2.5) == 2.5
        assert replicas.whole_job_rate(10.0, 1, 2.0) == 5.0
    finally:
        os.environ.update(env)


def _bench_reference(extra_env, tmp_path):
    env = dict(os.environ, **extra_env)
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "2048",
           "--steps", "1", "--warmup", "0", "--cpu-seconds", "0.2"]
    return subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=300,
                          cwd=str(tmp_path))


def test_reference_arm_other_ranks_exit_quietly(tmp_path):
    r = _bench_reference({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, tmp_path)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_reference_arm_rank0_prints_one_line(tmp_path):
    r = _bench_reference({"RANK": "0", "WORLD_SIZE": "2", "LOCAL_RANK": "0"}, tmp_path)
    assert r.returncode == 0, r.stderr[-500:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0


def test_cpu_baselines_all_cores_and_one_core():
    """bench.py's host-core baselines (the oracle port): the all-core rate
    and the one-core rate on a small Plummer sphere."""
    sys.path.insert(0, ROOT)
    import bench
    mass, pos, vel = bench.workload(1024)
    allc = bench.cpu_baseline(mass, pos, vel, 0.2, os.cpu_count() or 1)
    one = bench.single_core_baseline(mass, pos, vel, 0.5)
    assert allc["value"] > 0 and one["value"] > 0 and one["cores"] == 1
    assert allc["kind"] == "port" and "1 threads" in one["sample"]
