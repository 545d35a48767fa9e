"""The multi-GPU path of bench.py is replicas only (one independent solve per
rank, no data-path collective).  Its host-side logic, rendezvous, barrier and
the max-over-ranks aggregate of the per-rank solve times, runs here on CPU as
two gloo ranks."""
import json
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    w, r, local, dist = bench.dist_init()
    per_step = [1.0, 2.0, 3.0] if r == 0 else [4.0, 4.0, 4.0]   # rank 1 is the slow one
    bench.barrier(dist)
    value = bench.replica_value(dist, per_step, w)
    mx = bench.max_over_ranks(dist, float(r) + 0.5)
    bench.barrier(dist)
    with open(os.path.join(out_dir, f"rank{r}.json"), "w") as f:
        json.dump({"world": w, "rank": r, "local": local, "value": value, "max": mx}, f)
    dist.destroy_process_group()


def test_replica_aggregate_two_gloo_ranks(tmp_path):
    port = _free_port()
    mp.start_processes(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    for r, d in enumerate(res):
        assert d["world"] == 2 and d["rank"] == r and d["local"] == r
        # slowest rank's 12 ms over 2 ranks x 3 solves each
        assert d["value"] == pytest.approx(12.0 / 6)
        assert d["max"] == 1.5


def test_single_process_has_no_collective():
    sys.path.insert(0, ROOT)
    import bench

    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    w, r, local, dist = bench.dist_init()
    assert (w, r, local, dist) == (1, 0, 0, None)
    assert bench.replica_value(None, [2.0, 4.0], 1) == 3.0


def test_gpus_flag_starts_the_ranks_itself():
    """`bench.py --gpus 2` outside torchrun starts two ranks (torch.distributed.run
    on 127.0.0.1, gloo); the reference arm works on rank 0 only and prints one
    line whose n_gpus is the number of ranks that ran."""
    import subprocess

    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--size", "16",
                          "--steps", "1", "--warmup", "0", "--gpus", "2"], capture_output=True, text=True, env=env,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [json.loads(s) for s in out.stdout.splitlines() if s.startswith("{")]
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["ranks_with_work"] == 1
    assert d["rel_resid"] <= 1e-8 and d["steps"] == 1
