"""Multi-process (N > 1) host logic of bench.py on CPU, world size 2, gloo.

The transform does not shard ("replicas only"): every rank runs the same
workload and the job's time is the slowest rank's. These tests run the
aggregation and the rank handling the GPU path uses, without a GPU.
"""

import json
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


def _worker(rank: int, world: int, port: int, out_dir: str) -> None:
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, lr = bench.dist_env()
    ms = 10.0 + 5.0 * rank  # rank 1 is slower
    worst = bench.max_over_ranks(ms, w)
    dist.barrier()
    Path(out_dir, f"rank{rank}.json").write_text(json.dumps({"rank": r, "world": w, "local": lr, "max": worst}))
    dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    got = [json.loads((tmp_path / f"rank{i}.json").read_text()) for i in range(2)]
    assert [g["rank"] for g in got] == [0, 1] and all(g["world"] == 2 for g in got)
    assert all(g["max"] == 15.0 for g in got)  # both ranks report the slowest rank's time


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(3.5, 1) == 3.5


def test_reference_arm_only_rank0_prints(tmp_path):
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, env=env, cwd=str(ROOT), timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
