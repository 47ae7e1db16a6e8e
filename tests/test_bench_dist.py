"""Multi-process paths of bench.py on CPU (gloo): the path has no exchange between systems, so
N GPUs run N independent replicas ("replicas only"); the only cross-rank step is the max of the
timed milliseconds, and only rank 0 prints."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    v = bench.reduce_max(10.0 + 5.0 * rank, world)
    out[rank] = v
    dist.barrier()
    dist.destroy_process_group()


def test_reduce_max_gloo_two_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert dict(out) == {0: 15.0, 1: 15.0}


def test_reduce_max_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.reduce_max(3.5, 1) == 3.5


@pytest.mark.slow
def test_reference_arm_under_torchrun_prints_once():
    """`bench.py --impl reference` launched like the GPU arm (torchrun, 2 ranks): rank 0 alone runs
    the CPU reference port and prints one JSON line; the other rank exits 0."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
