"""bench.py's multi-rank path on CPU: world size 2 over gloo.

With N GPUs the bench runs one process per GPU, each tracking its own
replica of the workload (histories are independent: no data-path
collective), and reports the max over ranks of the timed durations and the
sum of the segments; rank 0 alone prints.  The reduction is exercised here
with two gloo ranks, and the reference arm under torchrun with two ranks
(rank 0 times the CPU port, the other rank exits at once)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, str(ROOT))
    import bench
    times, counts = bench.reduce_over_ranks(dist, [1.0 + rank, 5.0 - rank, 0.5], [100 + rank, 7], "cpu")
    dist.barrier()
    if rank == 0:
        Path(out_path).write_text(json.dumps({"times": times, "counts": counts}))
    dist.destroy_process_group()


def test_reduce_over_ranks_two_gloo_ranks(tmp_path):
    out = tmp_path / "reduced.json"
    torch.multiprocessing.spawn(_rank_main, args=(2, _free_port(), str(out)), nprocs=2, join=True)
    got = json.loads(out.read_text())
    assert got["times"] == [2.0, 5.0, 0.5]       # max over ranks
    assert got["counts"] == [201, 14]            # sum over ranks


def test_reduce_over_ranks_single_rank():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.reduce_over_ranks(None, [1.5, 2.0], [3, 4.0], "cpu") == ([1.5, 2.0], [3, 4])


def test_reference_arm_under_torchrun_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    res = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert res.returncode == 0, res.stderr[-3000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1                        # rank 0 alone prints
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
