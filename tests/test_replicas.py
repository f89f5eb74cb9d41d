"""The N > 1 path of bench.py on CPU, world size 2.

The library shards nothing (replicas only): under torchrun every rank runs
its own replica, the reported time is the slowest rank's (max over ranks),
and the reference arm runs on rank 0 alone while the other ranks exit 0.
These tests run that host logic with the gloo backend, no GPU involved.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, values, out_dir):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(dist, values[rank], "cpu")
    finally:
        dist.destroy_process_group()
    (Path(out_dir) / f"rank{rank}.txt").write_text(repr(got))


def test_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp

    values = [3.25, 7.5]
    mp.spawn(_rank_main, args=(2, _free_port(), values, str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        assert float((tmp_path / f"rank{r}.txt").read_text()) == max(values)


def test_reference_arm_prints_on_rank0_only():
    pytest.importorskip("numpy")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
