"""The multi-rank paths of bench.py on CPU: the step-time reduction over ranks
(gloo, world size 2) and the reference arm under torchrun, where rank 0 alone
measures and prints."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _reduce_worker(rank, world, port, values, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = bench.max_over_ranks(values[rank], dist, "cpu")
    finally:
        dist.destroy_process_group()


def test_step_time_is_the_slowest_rank():
    world = 2
    values = [3.25, 5.5]
    out = mp.Manager().dict()
    mp.spawn(_reduce_worker, args=(world, _free_port(), values, out), nprocs=world, join=True)
    assert dict(out) == {0: 5.5, 1: 5.5}


def test_weak_value_counts_every_rank():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.weak_value(2, 1000, 0.5) == 4000.0
    assert bench.max_over_ranks(1.5, None, "cpu") == 1.5


@pytest.mark.slow
def test_reference_arm_prints_once_under_torchrun():
    """Two ranks: rank 0 times the CPU restatement and prints one JSON line;
    rank 1 exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--log2n", "16"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0


def test_hbm_peak_is_the_measured_copy_rate():
    sys.path.insert(0, ROOT)
    import bench

    peak, src = bench.hbm_peak_gbs()
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            assert (peak, src) == (float(json.load(f)["hbm_gbs"]), "measured")
    else:
        assert (peak, src) == (bench.HBM_FALLBACK_GBS, "fallback")
