"""The bench's multi-GPU path (independent replicas, one process per GPU):
whole-job time is the slowest rank's and whole-job steps the sum over ranks.
Run here as two gloo processes on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, results):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r: 10 + r seconds, 1000 * (r + 1) steps
        results[rank] = bench.combine_ranks(dist, 10.0 + rank, 1000 * (rank + 1), "cpu")
    finally:
        dist.destroy_process_group()


def test_replica_time_is_the_max_and_steps_the_sum():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    world, port = 2, _free_port()
    with mp.Manager() as manager:
        results = manager.dict()
        procs = [mp.Process(target=_rank, args=(r, world, port, results)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs)
        for r in range(world):
            assert results[r] == (11.0, 3000.0)


def test_single_process_passes_through():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.combine_ranks(None, 2.5, 7, "cpu") == (2.5, 7.0)


def test_bench_launches_one_process_per_gpu():
    """`bench.py --gpus 2` started as a plain process launches two ranks
    (torch.distributed.run on 127.0.0.1) and rank 0 prints one line with
    n_gpus = 2.  --dry-run makes each rank report over gloo on the CPU instead
    of running the workload."""
    import json
    import subprocess
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT")}
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--dry-run"], capture_output=True,
                       text=True, timeout=180, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = lines[0]
    assert line["launcher_check"] is True
    assert line["n_gpus"] == 2 and line["requested_gpus"] == 2
    assert line["max_rank_seconds"] == 2.0 and line["sum_units"] == 3000.0


def test_served_summary_and_host_cpu():
    """The bench line's served-stream summary is taken from the served
    workload's own line (batched service against the plain path), and the CPU
    baseline names the host's CPU and core count."""
    sys.path.insert(0, ROOT)
    import bench
    serve = {"workload": "served_100: ...", "reply": "image",
             "plain": {"saturation_requests_per_s": 100.0, "load50": {"p50_ms": 12.0, "p99_ms": 40.0}},
             "batched": {"saturation_requests_per_s": 250.0, "lanes": 2, "load50": {"p50_ms": 10.0, "p99_ms": 30.0},
                         "at_plain_load50": {"p50_ms": 8.0, "p99_ms": 25.0}}}
    s = bench.served_summary(serve)
    assert s["workload"] == "served_100" and s["lanes"] == 2
    assert s["req_per_s"] == 250.0 and s["plain_req_per_s"] == 100.0 and s["ratio"] == 2.5
    assert (s["p50_ms"], s["p99_ms"], s["plain_p50_ms"], s["plain_p99_ms"]) == (10.0, 30.0, 12.0, 40.0)
    assert s["at_plain_load50"]["p50_ms"] == 8.0
    assert bench.served_summary(None) is None
    assert bench.served_summary({"error": "failed"}) is None
    cpu = bench.host_cpu()
    assert cpu["nproc"] == os.cpu_count() and isinstance(cpu["cpu_model"], str) and cpu["cpu_model"]
