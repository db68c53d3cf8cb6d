"""The multi-process (replica) path on CPU: world size 2 over gloo, 127.0.0.1 rendezvous.

A frame does not shard, so bench.py runs one replica per GPU and only combines timings: a
barrier, the maximum of the timed durations, the sum of per-replica rates. These tests run that
bookkeeping (rusterizer_gb300.replicas) in two processes, and the reference arm of bench.py
under torch.distributed.run, where rank 0 alone measures and prints."""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    from rusterizer_gb300.replicas import Replicas
    reps = Replicas("gloo", "cpu")
    reps.barrier()
    # rank r timed 10 + r ms and sustained 100 * (r + 1) requests/s with a p99 of 2 + r ms
    mx = reps.max([10.0 + rank, 2.0 + rank])
    sm = reps.sum([100.0 * (rank + 1)])
    reps.close()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"rank": reps.rank, "world": reps.world, "max": mx, "sum": sm}, f)


def test_replicas_max_and_sum_over_two_ranks(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, free_port(), str(tmp_path)), nprocs=world,
                       join=True, start_method="spawn")
    for r in range(world):
        res = json.load(open(tmp_path / f"rank{r}.json"))
        assert res["rank"] == r and res["world"] == world
        assert res["max"] == [11.0, 3.0]
        assert res["sum"] == [300.0]


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    from rusterizer_gb300.replicas import Replicas
    env = {k: os.environ.pop(k) for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK") if k in os.environ}
    try:
        reps = Replicas("gloo", "cpu")
        assert (reps.rank, reps.world, reps.pg) == (0, 1, None)
        assert reps.max([1.5, 2.5]) == [1.5, 2.5] and reps.sum([3.0]) == [3.0]
        reps.close()
    finally:
        os.environ.update(env)


def test_reference_arm_under_two_process_launch():
    """`bench.py --impl reference` launched like the multi-GPU bench: rank 0 prints exactly one
    JSON line, the other rank exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config", "0", "--steps", "1",
           "--warmup", "3"]
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["e2e"]["value"] == d["value"]
