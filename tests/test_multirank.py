"""The N > 1 paths of bench.py on the CPU with gloo and world size 2.

q-points are independent, so the bench shards them: rank r computes its own
q-point (no collective on the data path) and only the step time is reduced,
as the slowest rank's.  The reference arm runs on rank 0 alone while the
other ranks exit without work."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, queue):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    q = bench.q_steps_of_rank(rank)
    qs = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(qs, torch.tensor([q], dtype=torch.int64))
    slowest = bench.max_over_ranks(dist, 10.0 * rank + 1.0, device="cpu")
    queue.put((rank, [int(t.item()) for t in qs], slowest))
    dist.barrier()
    dist.destroy_process_group()


def test_q_sharding_and_slowest_rank_time():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(queue.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, qs, slowest in out:
        assert qs == [1, 2]          # one distinct q-point per rank
        assert slowest == 11.0       # the slowest rank's time on every rank


def test_ranks_compute_distinct_q_points(synth):
    sys.path.insert(0, ROOT)
    import bench
    qv = [synth.build(bench.config_of("small", bench.q_steps_of_rank(r))).q for r in range(2)]
    assert abs(qv[0] - qv[1]).max() > 0


def test_reference_arm_under_torchrun(orc):
    pytest.importorskip("torch")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--config", "small", "--cpu-budget", "1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1  # rank 0 alone prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
