"""Multi-process paths of bench.py on CPU (gloo): the path has no exchange between systems, so
N GPUs run N independent replicas of the single-system workload ("replicas only") and split the
batched ensembles by spin count; the only cross-rank steps are the max of the timed milliseconds
and the sum of the spins advanced, and only rank 0 prints."""
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


def test_partition_by_spins_balances_and_covers():
    """Every system lands on exactly one rank; the 256-system ensemble's spin loads differ by less
    than the largest system."""
    sys.path.insert(0, ROOT)
    import bench

    sizes = [sp["n_cells"][0] * sp["n_cells"][1] for sp in bench.c4_specs()]
    for world in (1, 2, 3, 4, 8):
        parts = bench.partition_by_spins(sizes, world)
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(len(sizes)))
        loads = [sum(sizes[k] for k in p) for p in parts]
        assert max(loads) - min(loads) <= max(sizes), (world, loads)
    assert bench.partition_by_spins([5, 3, 3, 1], 2) == [[0, 3], [1, 2]]


def _rank_sum_main(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    sizes = [sp["n_cells"][0] * sp["n_cells"][1] for sp in bench.c4_specs()]
    mine = bench.partition_by_spins(sizes, world)[rank]
    out[rank] = (bench.reduce_sum(sum(sizes[k] for k in mine), world), len(mine))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_spin_total_gloo_two_ranks():
    """Two gloo ranks shard the ensemble and sum their spins: both see the whole ensemble's count."""
    import torch.multiprocessing as mp

    sys.path.insert(0, ROOT)
    import bench

    total = sum(sp["n_cells"][0] * sp["n_cells"][1] for sp in bench.c4_specs())
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_sum_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0][0] == out[1][0] == total
    assert out[0][1] + out[1][1] == 256
