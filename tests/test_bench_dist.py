"""Multi-process paths of bench.py on CPU with the gloo backend (world size
2): the max-over-ranks timing helpers, and the reference arm launched under
torchrun, where rank 0 alone runs and prints one JSON line and the other
ranks exit 0 without work. The GPU arm's replicas use the same helpers over
NCCL; each replica advances its own mesh, with no collective in the step."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import argparse

    import torch.distributed as dist

    import bench
    w, r, _ = bench.dist_setup(argparse.Namespace(impl="reference"))
    assert (w, r) == (world, rank)
    bench.barrier(w)
    m = bench.allreduce_max(w, 1.5 + 2.0 * rank)
    with open(os.path.join(out_dir, "rank%d.txt" % rank), "w") as f:
        f.write(repr(m))
    dist.destroy_process_group()


def test_allreduce_max_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    mp.start_processes(_worker, args=(2, free_port(), str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        assert float((tmp_path / ("rank%d.txt" % r)).read_text()) == 3.5


def test_reference_arm_under_torchrun_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(free_port()), "bench.py", "--impl", "reference", "--gpus", "2",
           "--steps", "3", "--warmup", "3", "--workload", "sod_1st_inviscid_128x16x16"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["n_gpus"] == 2 and rec["value"] > 0
    assert rec["cpu_baseline"]["kind"] == "port" and rec["e2e"]["h2d_bytes_per_step"] == 0
