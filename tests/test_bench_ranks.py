"""The multi-GPU bench path is replicas only: rank results are combined as
the slowest rank's time and the summed scan length, and the reference arm
runs on rank 0 only.  Two gloo ranks on CPU."""

import os
import socket
import subprocess
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=2)
    import bench

    t = (10.0 + rank, 20.0 - rank)  # times: rank 1 slower on the value loop, rank 0 on e2e
    mm = (1.5 * (rank + 1), 2.5 * (rank + 1))
    res = bench.combine_ranks(t[0], t[1], mm[0], mm[1], torch.device("cpu"))
    out.put((rank, res))
    dist.barrier()
    dist.destroy_process_group()


def test_combine_ranks_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        assert got[r] == (11.0, 20.0, 4.5, 7.5)


def test_combine_ranks_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.combine_ranks(1.0, 2.0, 3.0, 4.0, torch.device("cpu")) == (1.0, 2.0, 3.0, 4.0)


@pytest.mark.parametrize("rank", [1])
def test_reference_arm_runs_on_rank_zero_only(rank):
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "1"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""  # the other ranks exit 0 without work or output


def test_reference_arm_line_on_rank_zero():
    """Rank 0 of the reference arm prints one JSON line with the GPU arm's
    metric, unit and config, the CPU sample described in cpu_baseline and an
    e2e block of the line's own value with no host-device bytes."""
    import json

    sys.path.insert(0, ROOT)
    import bench

    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [s for s in r.stdout.splitlines() if s.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 1
    assert d["metric"] == bench.METRIC and d["config"] == bench.bench_config(1)
    assert d["unit"] == "mm/s" and d["higher_is_better"] is True and d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
