"""The bench's multi-rank plumbing on CPU (gloo, world size 2): replicas launched by
torchrun, one JSON line from rank 0, max-over-ranks timing."""
import json
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


def _max_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    r, w = bench.dist_setup(world)
    bench.barrier(w)
    v = bench.max_over_ranks(float(10 + r), w)
    with open(os.path.join(out, f"r{r}.txt"), "w") as f:
        f.write(repr(v))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_max_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    assert [float(open(tmp_path / f"r{r}.txt").read()) for r in (0, 1)] == [11.0, 11.0]


def test_reference_arm_under_torchrun(oracle):
    """Two replicas: rank 0 alone runs and prints the reference line, rank 1 exits 0."""
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "small",
           "--gpus", "2", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["cpu_baseline"]["kind"] == "port" and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
