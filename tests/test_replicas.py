"""Multi-GPU is replicas only (independent evaluations, no collective on
the data path). CPU checks of the N > 1 paths of bench.py: the whole-job
rate over two gloo ranks (units summed, slowest rank's time), and the
reference arm under torch.distributed.run, where rank 0 alone prints."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench

    # rank r processed 100 * (r + 1) units in 2 * (r + 1) seconds
    rate = bench.replica_rate(100.0 * (rank + 1), 2.0 * (rank + 1), dist, "cpu")
    out[rank] = rate
    dist.destroy_process_group()


def test_replica_rate_over_two_gloo_ranks():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        rates = dict(out)
    # (100 + 200) units over the slowest rank's 4 s, the same on both ranks
    assert rates[0] == rates[1] == pytest.approx(75.0)


def test_reference_arm_under_torchrun_prints_once():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
           "--impl", "reference", "--gpus", "2", "--size", "24", "--patch", "2",
           "--candidates", "4", "--steps", "1", "--warmup", "1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0
