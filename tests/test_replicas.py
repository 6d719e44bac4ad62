"""The N > 1 path of bench.py on CPU (gloo, world size 2): replicas only, one grid per
rank, no data-path collective.  The timing reduction is the max over ranks, the value
all ranks' units over that time; under torchrun the reference arm runs on rank 0 alone
and prints one line."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, outdir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        ms = 100.0 + 50.0 * rank  # rank 1 is the slowest
        slow = bench.max_over_ranks(dist, ms, "cpu")
        value = bench.replica_value(world, 1000, 8, slow)
        with open(os.path.join(outdir, "%d.json" % rank), "w") as f:
            json.dump({"slowest": slow, "value": value}, f)
    finally:
        dist.destroy_process_group()


def test_replica_reduction_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = free_port()
    mp.spawn(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    res = [json.load(open(tmp_path / ("%d.json" % r))) for r in range(2)]
    for r in res:
        assert r["slowest"] == 150.0  # every rank sees the slowest rank's time
        assert r["value"] == pytest.approx(2 * 1000 * 8 / 0.150, rel=1e-15)


def test_replica_helpers_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(None, 3.5, "cpu") == 3.5
    assert bench.replica_value(1, 1048576, 8, 1000.0) == pytest.approx(8 * 1048576, rel=1e-15)


def test_reference_arm_under_torchrun_prints_one_line():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "4", "--warmup", "1", "--nx", "128", "--ny", "64"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0
