"""The N > 1 launch path of bench.py on CPU: world size 2 over gloo.

The event loop of one system is sequential, so N GPUs run N independent
replicas ("replicas only"): the only cross-rank traffic is the max / sum of the
timing and event counts.  These tests run two gloo ranks on the host.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": "2", "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, REPO)
    import bench
    D = bench.Dist()
    out[rank] = (D.max(float(rank + 1)), D.sum(float(10 * (rank + 1))))
    D.barrier()
    D.td.destroy_process_group()


def test_dist_max_and_sum_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    port = free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(port, out), nprocs=2, join=True)
        assert dict(out) == {0: (2.0, 30.0), 1: (2.0, 30.0)}


def test_reference_arm_under_torchrun_prints_one_line_from_rank_0():
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "3", "--workload", "c1", "--cpu-seconds", "0.5"]
    r = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0
