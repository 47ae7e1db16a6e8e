#!/usr/bin/env python
"""Benchmark: spin-updates/s of LLG with dipolar interaction on one GB300.

Workload (one "step" = one stochastic Heun iteration of the whole system, both predictor and
corrector stages, each with the full dipolar FFT convolution):
    simple cubic 128 x 128 x 16, lattice constant 4 Angstrom, mu_s = 2 mu_B, J = 1 meV (nearest
    neighbours), bulk (Bloch) DMI D = 0.2 meV, uniaxial K = 0.05 meV along z, B_z = 0.5 T,
    periodic in a and b, open in c; dipole-dipole by zero-padded FFT (padding along c only:
    the "2N" padded volume 128 x 128 x 32, 4 periodic images in a and b);
    T = 10 K (Philox thermal noise), alpha = 0.1, dt = 5e-4 ps, FP32 bulk arithmetic.
Inputs are seeded random unit spins; the device timing flushes L2 before every timed step
(writes a 512 MiB buffer, then reads another 512 MiB so the write-back of the dirty flush lines
is not charged to the step), because the working set (~35 MB) would otherwise stay in the
129 MB L2.

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Under torchrun every rank runs an independent replica (the path has no exchange between
systems: "replicas only"); rank 0 prints one JSON line.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "spin-updates/s LLG+dipolar, batched vs plain on 1 GB300 at max|Δm|<=1e-5; vs CPU"
N_CELLS = [128, 128, 16]
SPEC = dict(
    bravais="sc", n_cells=N_CELLS, lattice_constant=4.0, mu_s=[2.0], bc=[1, 1, 0],
    field=(0.5, (0, 0, 1)), anisotropy=(0.05, (0, 0, 1)), jij=[1.0], dij=[0.2], dm_chirality=1,
    ddi=dict(method="fft", n_periodic_images=[4, 4, 0], radius=0.0, pb_zero_padding=0),
    llg=dict(dt=5e-4, damping=0.1, temperature=10.0, seed=2, force_convergence=1e-10),
)
NOS = N_CELLS[0] * N_CELLS[1] * N_CELLS[2]
CONFIG = {
    "workload": "SC 128x128x16 LLG stochastic Heun T=10K + DDI FFT (2N z-padding), FP32 bulk",
    "n_spins": NOS, "solver": "Heun", "dt_ps": 5e-4, "alpha": 0.1, "temperature_K": 10.0,
    "ddi_padded_extent": [128, 128, 32],
    "l2": "flushed before every timed step (512 MiB write, then 512 MiB read)",
}
KERNELS = ["stage", "fft_pass_a", "fft_pass_b", "fft_pass_c_tensor", "fft_pass_b_inv", "fft_pass_a_inv_c2r", "",
           "fft_pass_bc_tensor"]


def algorithmic_bytes(kernel, stage, rows=False):
    """Algorithmic HBM bytes of one launch at the workload size, FP32 (SoA spins 12 B/spin,
    complex 8 B).  Stage 1 of Heun reads s and h, writes predictor and fv1 (48 B/spin); stage 2
    reads predictor, s, fv1, h and writes s (60 B/spin).  FFT passes read and write their
    half-spectrum arrays once; pass C also reads the 6-component dipole spectrum.  Row-fused
    stages (rows=True) read the field spectrum and write the next configuration's instead of
    reading h: stage bytes - 12 B/spin + 2 W1."""
    Mh, Mb, Mc, Nb, Nc = 65, 128, 32, 128, 16
    W1 = 3 * Nc * Nb * Mh * 8
    W2 = 3 * Nc * Mb * Mh * 8
    D = 6 * Mc * Mb * Mh * 8
    S = 12 * NOS
    return {
        "stage": (48 if stage == 1 else 60) * NOS + ((2 * W1 - 12 * NOS) if rows else 0),
        "fft_pass_a": S + W1,
        "fft_pass_b": W1 + W2,
        "fft_pass_c_tensor": 2 * W2 + D,
        "fft_pass_b_inv": W2 + W1,
        "fft_pass_a_inv_c2r": W1 + S,
        # fused b/c pass: W1 in and out, the dipole spectrum once
        "fft_pass_bc_tensor": 2 * W1 + D,
    }[kernel]


# DRAM bytes (read + write) per launch of the dominant kernels on this workload, from the committed
# summaries of one ncu capture each (profiles/<file>: a line "dram_bytes_per_launch: N")
TRAFFIC_PROFILES = {"fft_pass_bc_tensor": "fft_pass_bc_cl_sc128x128x16_dram.md",
                    "stage": "llg_stage_heun_sc128x128x16_dram.md"}


def profiled_traffic(kernel):
    """dram__bytes_read.sum + dram__bytes_write.sum per launch of `kernel` from its profile summary
    under profiles/, or None when there is none."""
    name = TRAFFIC_PROFILES.get(kernel)
    if not name:
        return None
    try:
        with open(os.path.join(ROOT, "profiles", name)) as f:
            for line in f:
                if line.strip().startswith("dram_bytes_per_launch:"):
                    return int(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 6:
                continue
            try:
                sm.append(float(p[0]))
                smax = max(smax, float(p[1]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if p[2 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_max(v, world):
    """Max over the ranks of one number (the timed region's milliseconds): every rank runs its own
    replica, the slowest one sets the job time."""
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline(seconds=12.0):
    """The oracle (CPU FP64 restatement of the reference path, OpenMP over all host cores) on a
    bounded sample of the same workload: as many Heun steps as fit in ~`seconds`."""
    from oracle.oracle import OracleSystem, random_spins

    o = OracleSystem(SPEC)
    s0 = random_spins(NOS, 1)
    t0 = time.perf_counter()
    o.llg(s0, "Heun", 1, dt=5e-4, damping=0.1, temperature=10.0, seed=2)
    t1 = time.perf_counter() - t0
    n = max(1, min(40, int(seconds / max(t1, 1e-3))))
    t0 = time.perf_counter()
    o.llg(s0, "Heun", n, dt=5e-4, damping=0.1, temperature=10.0, seed=2)
    dt = time.perf_counter() - t0
    return {"value": NOS * n / dt, "unit": "spin-updates/s", "cores": os.cpu_count(), "kind": "port",
            "sample": "%d stochastic Heun steps of the full 128x128x16 DDI system (FP64, OpenMP)" % n}


def c2_accuracy(steps=200):
    """Accuracy of the headline workload: the device FP32 path and the FP64 oracle run `steps`
    stochastic Heun steps of the full 128x128x16 dipolar system from the same seeded spins,
    drawing the same Philox stream (seed 2, stream 0); max |dm| over all spins.  Outside the
    timed region."""
    from oracle.oracle import OracleSystem, random_spins
    from spirit_gb300 import simulation, state, system
    from spirit_gb300.configs import write_config

    s0 = random_spins(NOS, 1)
    p = state.setup(write_config(SPEC, os.path.join(tempfile.mkdtemp(), "acc.cfg")), True)
    system.get_spin_directions(p)[:] = s0
    simulation.set_precision(p, 32)
    simulation.start(p, simulation.METHOD_LLG, simulation.SOLVER_HEUN, steps)
    got = np.array(system.get_spin_directions(p))
    state.delete(p)
    ref, _ = OracleSystem(SPEC).llg(s0, "Heun", steps, dt=5e-4, damping=0.1, temperature=10.0, seed=2, stream=0)
    return {"steps": steps, "max_dm_vs_fp64_oracle": float(np.abs(got - ref).max()),
            "check": "headline workload (T=10 K, same Philox stream), FP32 device vs FP64 oracle"}


def cufft_comparison(ddi_ms_per_eval, iters=30):
    """Timing yardstick for the hand-written dipolar passes (timing only, never a product path):
    the same field evaluation of the headline system -- R2C of mu*s on the zero-padded 128x128x32
    volume, the 6-component symmetric tensor product, C2R -- with cuFFT through torch.fft (3 batched
    transforms each way) and the product as torch elementwise ops, FP32, L2 flushed before every
    evaluation, CUDA events.  The hand-written path is passes A, b/c (transforms along b and c and
    the product fused) and A' per evaluation, from the per-kernel profile."""
    import torch

    Na, Nb, Nc, Mc = 128, 128, 16, 32
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn(3, Nc, Nb, Na, device="cuda", generator=g)
    Dh = torch.randn(6, Mc, Nb, Na // 2 + 1, 2, device="cuda", generator=g)
    Dh = torch.view_as_complex(Dh)
    flush = torch.empty(512 * 2**20, dtype=torch.uint8, device="cuda")
    t_fft, t_all = [], []
    for it in range(iters + 3):
        flush.fill_(it & 0xFF)
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        e[0].record()
        X = torch.fft.rfftn(x, s=(Mc, Nb, Na), dim=(1, 2, 3))
        e[1].record()
        H = torch.stack([Dh[0] * X[0] + Dh[1] * X[1] + Dh[2] * X[2],
                         Dh[1] * X[0] + Dh[3] * X[1] + Dh[4] * X[2],
                         Dh[2] * X[0] + Dh[4] * X[1] + Dh[5] * X[2]])
        e[2].record()
        h = torch.fft.irfftn(H, s=(Mc, Nb, Na), dim=(1, 2, 3))[:, :Nc]
        e[3].record()
        torch.cuda.synchronize()
        if it >= 3:
            t_fft.append(e[0].elapsed_time(e[1]) + e[2].elapsed_time(e[3]))
            t_all.append(e[0].elapsed_time(e[3]))
    del h
    return {"cufft_transforms_ms": statistics.median(t_fft), "cufft_with_torch_product_ms": statistics.median(t_all),
            "handwritten_ms": ddi_ms_per_eval,
            "handwritten_vs_cufft_transforms": statistics.median(t_fft) / ddi_ms_per_eval if ddi_ms_per_eval else None,
            "what": "one dipolar field evaluation of the 128x128x16 system (padded 128x128x32), FP32"}


def run_reference(args):
    """The reference arm: the CPU port of the reference path (oracle/, FP64, OpenMP on all host
    cores) on the same workload; one step = one stochastic Heun iteration of the full system.
    The set-up (neighbours, dipole spectrum) is outside the timed region, as in the reference."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle.oracle import OracleSystem, random_spins

    o = OracleSystem(SPEC)
    s = random_spins(NOS, 1)
    if args.warmup > 0:
        s, _ = o.llg(s, "Heun", args.warmup, dt=5e-4, damping=0.1, temperature=10.0, seed=2)
    t0 = time.perf_counter()
    s, _ = o.llg(s, "Heun", args.steps, dt=5e-4, damping=0.1, temperature=10.0, seed=2)
    dt = time.perf_counter() - t0
    v = NOS * args.steps / dt
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "spin-updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded random spins)", "config": CONFIG,
        "cpu_baseline": {"value": v, "unit": "spin-updates/s", "cores": cores, "kind": "port",
                         "sample": "%d stochastic Heun steps of the full 128x128x16 DDI system (FP64, OpenMP, "
                                   "%d threads)" % (args.steps, cores)},
        "e2e": {"value": v, "unit": "spin-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def partition_by_spins(sizes, world):
    """Shard independent systems over `world` ranks by spin count (no exchange between systems):
    largest first, each to the rank with the fewest spins so far (ties: the lowest rank).  Returns
    one list of system indices per rank, each in ascending order."""
    load = [0] * world
    parts = [[] for _ in range(world)]
    for k in sorted(range(len(sizes)), key=lambda k: (-sizes[k], k)):
        r = min(range(world), key=lambda r: (load[r], r))
        parts[r].append(k)
        load[r] += sizes[k]
    return [sorted(p) for p in parts]


def reduce_sum(v, world):
    """Sum over the ranks of one number (the spins each rank advanced)."""
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def c4_specs(n=256, seed=4, ddi=False):
    """The batched uneven ensemble: n periodic square lattices with edge lengths log-uniform in
    [32, 256] and per-system J, D (Neel), K, B_z, T drawn from the given seed; SIB, alpha 0.2,
    dt 1e-3 ps, mu_s 2 mu_B.  ddi=True: the dipolar variant -- open boundaries, DDI by FFT
    (zero-padded 2L x 2L, no periodic images), lattice constant 4 A."""
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(n):
        L = int(round(np.exp(rng.uniform(np.log(32), np.log(256)))))
        J, D, K = rng.uniform(0.5, 1.5), rng.uniform(0.0, 0.4), rng.uniform(0.0, 0.2)
        B, T = rng.uniform(0.0, 2.0), rng.uniform(0.0, 50.0)
        sp = dict(bravais="sc", n_cells=[L, L, 1], lattice_constant=1.0, mu_s=[2.0], bc=[1, 1, 0],
                  field=(B, (0, 0, 1)), anisotropy=(K, (0, 0, 1)), jij=[J], dij=[D], dm_chirality=2,
                  llg=dict(dt=1e-3, damping=0.2, temperature=T, seed=1000 + k))
        if ddi:
            sp.update(bc=[0, 0, 0], lattice_constant=4.0,
                      ddi=dict(method="fft", n_periodic_images=[0, 0, 0], radius=0.0, pb_zero_padding=1))
        specs.append(sp)
    return specs


def run_batched_vs_plain(steps, warmup, plain=True, check=True, ddi=False, profile_step=False, n_systems=256):
    """256 uneven systems: spin-updates/s of the batched path (all systems in one launch per SIB
    stage, CUDA graphs) against the plain path (every system its own engine and launches, on the
    same stream), both FP32 and device-timed with CUDA events; the ensemble's arrays (~290 MB)
    exceed L2.  Accuracy: the 8 smallest systems run 1000 batched FP32 steps against the FP64
    oracle consuming the same Philox streams.  ddi=True: the dipolar variant of the ensemble
    (c4_specs), one batched FFT plan over all 256 systems.  profile_step: one more batched step
    inside a profiler range (for `ncu --profile-from-start off`).  n_systems: the first n systems of
    the ensemble (the same seeds), for profiler captures on a small case."""
    import torch

    from oracle.oracle import OracleSystem, random_spins
    from spirit_gb300 import simulation, state, system
    from spirit_gb300.configs import write_config
    from spirit_gb300.spiritlib import fn

    launch = fn("Simulation_Launch_Steps", [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int])
    rank, world, _ = dist_env()
    specs = c4_specs(n=n_systems, ddi=ddi)
    if world > 1:
        # the ensemble is sharded over the ranks by spin count; each rank batches its share
        mine = partition_by_spins([sp["n_cells"][0] * sp["n_cells"][1] for sp in specs], world)[rank]
        specs = [specs[k] for k in mine]
    tmp = tempfile.mkdtemp()
    states, nos = [], []
    for k, sp in enumerate(specs):
        p = state.setup(write_config(sp, os.path.join(tmp, "c4_%d.cfg" % k)), True)
        n = sp["n_cells"][0] * sp["n_cells"][1]
        system.get_spin_directions(p)[:] = random_spins(n, 4000 + k)
        simulation.set_precision(p, 32)
        states.append(p)
        nos.append(n)
    total = sum(nos)
    stream = torch.cuda.Stream()
    for p in states:
        simulation.set_stream(p, stream.cuda_stream)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    # plain: one engine and one launch sequence per system
    plain_ms = float("nan")
    for p in (states if plain else []):
        simulation.start(p, simulation.METHOD_LLG, simulation.SOLVER_SIB, 10**9, -1, True)
    if plain:
        for _ in range(warmup):
            for p in states:
                launch(p, 1, -1, -1)
        stream.synchronize()
        a, b = ev(), ev()
        a.record(stream)
        for _ in range(steps):
            for p in states:
                launch(p, 1, -1, -1)
        b.record(stream)
        stream.synchronize()
        plain_ms = a.elapsed_time(b)
        for p in states:
            simulation.stop(p)
    # batched: all systems in one engine
    simulation.batched_launch_steps(states, simulation.SOLVER_SIB, warmup)
    stream.synchronize()
    a, b = ev(), ev()
    a.record(stream)
    simulation.batched_launch_steps(states, simulation.SOLVER_SIB, steps)
    b.record(stream)
    stream.synchronize()
    batched_ms = a.elapsed_time(b)
    if profile_step:
        torch.cuda.profiler.start()
        simulation.batched_launch_steps(states, simulation.SOLVER_SIB, 1)
        stream.synchronize()
        torch.cuda.profiler.stop()
    simulation.batched_finish(states)
    for p in states:
        state.delete(p)
    # accuracy after 1000 steps: 8 smallest systems in fresh States (Philox streams from their
    # start), batched FP32 vs the FP64 oracle
    small = sorted(range(len(specs)), key=lambda k: nos[k])[:8 if check else 0]
    sub = []
    s0 = [random_spins(nos[k], 5000 + k) for k in small]
    for k, s in zip(small, s0):
        p = state.setup(write_config(specs[k], os.path.join(tmp, "c4_%d.cfg" % k)), True)
        system.get_spin_directions(p)[:] = s
        simulation.set_precision(p, 32)
        sub.append(p)
    if sub:
        simulation.start_batched(sub, simulation.SOLVER_SIB, 1000)
    dm = 0.0 if sub else None
    for j, k in enumerate(small):
        sp = specs[k]
        o = OracleSystem(sp)
        ref, _ = o.llg(s0[j], "SIB", 1000, dt=1e-3, damping=0.2, temperature=sp["llg"]["temperature"],
                       seed=sp["llg"]["seed"], stream=j)
        got = np.array(system.get_spin_directions(sub[j]))
        dm = max(dm, float(np.abs(got - ref).max()))
    for p in sub:
        state.delete(p)
    if dm is not None:
        dm = reduce_max(dm, world)
    # whole-job rates: the spins of every rank over the slowest rank's time
    all_spins = reduce_sum(total, world)
    batched_ms = reduce_max(batched_ms, world)
    plain_ms = reduce_max(plain_ms, world) if plain else plain_ms
    bv = all_spins * steps / (batched_ms / 1000.0)
    pv = all_spins * steps / (plain_ms / 1000.0)
    n_all = int(reduce_sum(len(specs), world))
    if ddi:
        workload = ("%d uneven open SC 2D systems with the dipolar interaction (DDI FFT, zero-padded 2L x 2L, "
                    "a = 4 A), L log-uniform in [32,256] (seed 4), per-system J, D, K, B_z, T in U[0,50] K; "
                    "stochastic SIB alpha=0.2 dt=1e-3 ps, FP32" % n_all)
        plain_desc = "one engine per system (its own FFT plan), 2 stages x (DDI passes + stage) per step, same stream"
    else:
        workload = ("%d uneven periodic SC 2D systems, L log-uniform in [32,256] (seed 4), per-system J, D, K, "
                    "B_z, T in U[0,50] K; stochastic SIB alpha=0.2 dt=1e-3 ps, FP32" % n_all)
        plain_desc = "one engine per system, 2 launches per system per step (1-step CUDA graph), same stream"
    arrays_mb = total * 72 / 1e6
    l2_note = ("not flushed: the ensemble's 6 x 3 FP32 arrays (%.0f MB) %s the 129 MB L2"
               % (arrays_mb, "exceed" if arrays_mb > 129 else "fit in (a small profiling case)"))
    return {
        "workload": workload,
        "n_systems": n_all, "n_spins": int(all_spins), "steps": steps, "warmup": warmup,
        "sharding": "systems split over %d ranks by spin count" % world if world > 1 else "one rank",
        "value": bv, "unit": "spin-updates/s", "ms_per_step": batched_ms / steps,
        "plain_value": pv, "plain_ms_per_step": plain_ms / steps, "ratio_batched_vs_plain": bv / pv,
        "plain": plain_desc,
        "l2": l2_note,
        "max_dm_vs_fp64_oracle": dm,
        "accuracy_check": "8 smallest systems, 1000 batched FP32 steps vs the FP64 oracle on the same Philox streams",
    }


def compact_batched(v):
    """The batched-vs-plain figures the metric names, in a few keys (the end of the JSON line)."""
    return {"ratio": v["ratio_batched_vs_plain"], "batched_value": v["value"], "plain_value": v["plain_value"],
            "unit": v["unit"], "ms_per_step": v["ms_per_step"], "plain_ms_per_step": v["plain_ms_per_step"],
            "n_systems": v["n_systems"], "n_spins": v["n_spins"], "steps": v["steps"],
            "max_dm_vs_fp64_oracle": v["max_dm_vs_fp64_oracle"], "accuracy_steps": 1000}


C3_SPEC = dict(bravais="hex2d60", n_cells=[96, 96, 1], lattice_constant=1.0, mu_s=[2.0], bc=[1, 1, 0],
               field=(1.5, (0, 0, 1)), anisotropy=(0.08, (0, 0, 1)), jij=[1.0], dij=[0.35], dm_chirality=2,
               llg=dict(dt=1e-3, damping=0.3, temperature=0.0),
               gneb=dict(spring_constant=1.0, force_convergence=1e-6))
C3_IMAGES = 32


def neel_skyrmion(pos, center, radius=8.0, width=2.0, sign=1.0):
    """Neel skyrmion with the tanh profile theta(rho) = pi/2 (1 - tanh((rho - R) / w)), core down at
    `center`; sign picks the radial sense of the in-plane component."""
    d = pos[:, :2] - np.asarray(center)[:2]
    rho = np.hypot(d[:, 0], d[:, 1])
    th = 0.5 * np.pi * (1.0 - np.tanh((rho - radius) / width))
    phi = np.arctan2(d[:, 1], d[:, 0])
    return np.stack([sign * np.sin(th) * np.cos(phi), sign * np.sin(th) * np.sin(phi), np.cos(th)], axis=1)


def run_gneb(iters_cap=60000):
    """Batched GNEB: 32 images of a 96x96 triangular lattice between a relaxed Neel skyrmion
    (radius 8 sites) and the ferromagnet (geodesic interpolation), spring 1, VP; 2000 plain
    iterations, then climbing / falling images set automatically and iterations until the max
    torque is below 1e-5 meV with FP32 forces, then FP64 forces to 1e-6 meV (or the cap); FP64
    energies."""
    from oracle.oracle import OracleSystem
    from spirit_gb300 import chain, geometry, simulation, state, system, transition
    from spirit_gb300.configs import write_config
    import spirit_gb300.parameters.gneb as gneb
    import spirit_gb300.parameters.llg as llg

    p = state.setup(write_config(C3_SPEC, os.path.join(tempfile.mkdtemp(), "c3.cfg")), True)
    simulation.set_precision(p, 32)
    pos = np.array(geometry.get_positions(p))
    center = 0.5 * (pos.min(axis=0) + pos.max(axis=0))
    best = None
    for sign in (1.0, -1.0):
        system.get_spin_directions(p)[:] = neel_skyrmion(pos, center, sign=sign)
        e = system.get_energy_fp64(p)
        if best is None or e < best[0]:
            best = (e, sign)
    system.get_spin_directions(p)[:] = neel_skyrmion(pos, center, sign=best[1])
    # the skyrmion endpoint relaxed in FP64 by L-BFGS to 1e-9 meV (the barrier is measured from its
    # energy; a softer convergence leaves the breathing mode under-relaxed by ~1e-5 meV)
    simulation.set_precision(p, 64)
    llg.set_convergence(p, 1e-9)
    simulation.start(p, simulation.METHOD_LLG, simulation.SOLVER_LBFGS_OSO, 20000)
    simulation.set_precision(p, 32)
    sk = np.array(system.get_spin_directions(p))
    nos = sk.shape[0]
    chain.image_to_clipboard(p)
    for _ in range(1, C3_IMAGES):
        chain.insert_image_after(p)
    system.get_spin_directions(p, 0)[:] = sk
    fm = np.zeros_like(sk)
    fm[:, 2] = 1.0
    system.get_spin_directions(p, C3_IMAGES - 1)[:] = fm
    transition.homogeneous(p, 0, C3_IMAGES - 1)
    gneb.set_convergence(p, 1e-6)
    gneb.set_spring_constant(p, 1.0)
    chain0 = np.array([np.array(system.get_spin_directions(p, i)) for i in range(C3_IMAGES)])
    # FP32 forces until the max torque is below 1e-5 meV (FP32 rounding of the forces leaves a torque
    # floor of a few 1e-6 meV), then FP64 to the 1e-6 meV criterion from the same chain and image types
    t0 = time.perf_counter()
    gneb.set_convergence(p, 1e-5)
    info1 = simulation.start(p, simulation.METHOD_GNEB, simulation.SOLVER_VP, 2000)
    gneb.set_image_type_automatically(p)
    info2 = simulation.start(p, simulation.METHOD_GNEB, simulation.SOLVER_VP, iters_cap)
    t1 = time.perf_counter()
    it32 = int(info1.total_iterations) + int(info2.total_iterations)
    mt32 = float(info2.max_torque)
    E32 = np.array([system.get_energy_fp64(p, i) for i in range(C3_IMAGES)])
    simulation.set_precision(p, 64)
    gneb.set_convergence(p, 1e-6)
    info3 = simulation.start(p, simulation.METHOD_GNEB, simulation.SOLVER_VP, iters_cap)
    t2 = time.perf_counter()
    it64 = int(info3.total_iterations)
    mt = float(info3.max_torque)
    E = np.array([system.get_energy_fp64(p, i) for i in range(C3_IMAGES)])
    chain1 = np.array([np.array(system.get_spin_directions(p, i)) for i in range(C3_IMAGES)])
    types = np.array([gneb.get_climbing_falling(p, i) for i in range(C3_IMAGES)])
    state.delete(p)
    n_it = it32 + it64
    spins = C3_IMAGES * nos
    # the oracle (FP64 CPU restatement) continued from the device's converged chain with the same image
    # types: its barrier and max torque after a bounded number of iterations
    o = OracleSystem(C3_SPEC)
    _, ro = o.gneb(chain1, 50, image_type=types, spring_constant=1.0, force_convergence=1e-12, dt=1e-3)
    Eo = np.asarray(ro["energies"])
    # CPU: the oracle's GNEB iteration (FP64, OpenMP) on the same chain, a bounded sample
    n_cpu = 3
    c0 = time.perf_counter()
    o.gneb(chain0, n_cpu, spring_constant=1.0, force_convergence=1e-6, dt=1e-3)
    cpu_s = time.perf_counter() - c0
    return {
        "workload": "GNEB, 32 images of a periodic 96x96 triangular lattice (J=1, Neel D=0.35, K=0.08 meV, "
                    "B=1.5 T), relaxed Neel skyrmion (R=8 sites, tanh profile; FP64 L-BFGS to 1e-9) to ferromagnet, spring 1, VP, "
                    "climbing image after 2000 iterations, convergence 1e-6 meV; FP32 forces to 1e-5 meV, then "
                    "FP64 forces to 1e-6 meV; FP64 energies",
        "n_images": C3_IMAGES, "spins_per_image": nos,
        "iterations": n_it, "iterations_fp32": it32, "iterations_fp64": it64, "converged": bool(mt < 1e-6),
        "max_torque": mt, "max_torque_after_fp32": mt32,
        "wall_s": t2 - t0, "wall_s_fp32": t1 - t0, "ms_per_iteration": 1000.0 * (t2 - t0) / n_it,
        "value": spins * n_it / (t2 - t0), "unit": "spin-updates/s",
        "barrier_meV": float(E.max() - E[0]), "barrier_meV_after_fp32": float(E32.max() - E32[0]),
        "saddle_image": int(E.argmax()),
        "oracle_check": {"iterations": 50, "barrier_meV": float(Eo.max() - Eo[0]),
                         "max_torque": float(ro["max_torque"]),
                         "what": "FP64 oracle GNEB continued from the converged device chain (same image types)"},
        "timing": "wall clock of the three Simulation_GNEB_Start calls (host checks between device chunks included)",
        "cpu_baseline": {"value": spins * n_cpu / cpu_s, "unit": "spin-updates/s", "cores": os.cpu_count(),
                         "kind": "port", "sample": "%d GNEB iterations of the same 32-image chain (FP64, OpenMP)" % n_cpu},
    }


C5_SPEC = dict(bravais="sc", n_cells=[128, 128, 1], lattice_constant=1.0, mu_s=[2.0], bc=[0, 0, 0],
               field=(0.8, (0, 0, 1)), anisotropy=(0.1, (0, 0, 1)), jij=[1.0], dij=[0.3], dm_chirality=2,
               ddi=dict(method="fft", n_periodic_images=[0, 0, 0], radius=0.0, pb_zero_padding=1),
               llg=dict(dt=1e-3, damping=0.3, temperature=0.0))


def run_adjoint(n_steps=2000, checkpoint=100):
    """Adjoint workload: 128x128 open square lattice with padded dipolar FFT (256x256), RK4
    dt=1e-3 ps, 2000 steps, loss = mean |s(T) - target|^2 against a seeded target; gradient with
    respect to s0 and (J, D, K, B_z, alpha) by the hand-written adjoint, checkpoint every 100 steps.
    Forward and adjoint wall times exclude the shared set-up (measured as a 0-step call)."""
    from oracle.oracle import random_spins
    from spirit_gb300 import adjoint, simulation, state, system
    from spirit_gb300.configs import write_config

    p = state.setup(write_config(C5_SPEC, os.path.join(tempfile.mkdtemp(), "c5.cfg")), True)
    simulation.set_precision(p, 32)
    nos = 128 * 128
    system.get_spin_directions(p)[:] = random_spins(nos, 55)
    tgt = random_spins(nos, 56)
    prm = np.array([1.0, 0.3, 0.1, 0.8, 0.3])
    adjoint.llg_loss(p, tgt, 2, prm)  # warm-up (module loading)
    adjoint.llg_adjoint(p, tgt, 2, 1, prm)  # builds the second dipolar lane of the pipelined backward pass
    t0 = time.perf_counter()
    adjoint.llg_loss(p, tgt, 0, prm)
    setup_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    loss_f, _ = adjoint.llg_loss(p, tgt, n_steps, prm)
    fwd_s = time.perf_counter() - t0 - setup_s
    t0 = time.perf_counter()
    loss_a, g0, gp, _ = adjoint.llg_adjoint(p, tgt, n_steps, checkpoint, prm)
    adj_s = time.perf_counter() - t0 - setup_s
    # the whole trajectory recorded in HBM (16 stage arrays per step): no recomputation
    t0 = time.perf_counter()
    loss_r, g0_r, gp_r, _ = adjoint.llg_adjoint(p, tgt, n_steps, n_steps, prm)
    rec_s = time.perf_counter() - t0 - setup_s
    state.delete(p)
    rec_bytes = n_steps * 16 * 3 * nos * 4
    return {
        "workload": "adjoint of RK4 LLG: 128x128 open SC 2D, DDI FFT padded 256x256, J=1, D=0.3, K=0.1 meV, "
                    "B=0.8 T, alpha=0.3, dt=1e-3 ps, %d steps, checkpoint %d; FP32 forward and adjoint, FP64 loss"
                    % (n_steps, checkpoint),
        "n_spins": nos, "steps": n_steps, "forward_s": fwd_s, "adjoint_s": adj_s,
        "adjoint_over_forward": adj_s / fwd_s,
        "full_record": {"checkpoint": n_steps, "adjoint_s": rec_s, "adjoint_over_forward": rec_s / fwd_s,
                        "recorded_bytes": rec_bytes,
                        "max_abs_diff_grad_s0": float(np.max(np.abs(np.asarray(g0_r) - np.asarray(g0)))),
                        "max_abs_diff_grad_params": float(np.max(np.abs(np.asarray(gp_r) - np.asarray(gp)))),
                        "loss": loss_r},
        "forward_value": nos * n_steps / fwd_s, "unit": "spin-updates/s", "setup_s": setup_s,
        "loss": loss_a, "loss_forward_only": loss_f,
        "grad_params": {k: float(v) for k, v in zip(adjoint.PARAMS, gp)},
        "timing": "wall clock of Simulation_LLG_Loss / Simulation_LLG_Adjoint minus a 0-step call (engine set-up)",
    }


def run_mc(sweeps=200):
    """Monte Carlo on the C2 lattice (SC 128x128x16; the single-spin energy has no dipolar term):
    Metropolis sweeps at T = 10 K with the adaptive cone, FP32, timed by wall clock around
    Simulation_MC_Start after a warm-up run; CPU: the oracle's sweep (FP64, OpenMP) on a sample."""
    from oracle.oracle import OracleSystem, random_spins
    from spirit_gb300 import simulation, state, system
    from spirit_gb300.configs import write_config
    import spirit_gb300.parameters.mc as mc

    spec = dict(SPEC)
    spec.pop("ddi", None)
    p = state.setup(write_config(spec, os.path.join(tempfile.mkdtemp(), "mc.cfg")), True)
    simulation.set_precision(p, 32)
    system.get_spin_directions(p)[:] = random_spins(NOS, 5)
    mc.set_temperature(p, 10.0)
    simulation.start(p, simulation.METHOD_MC, n_iterations=16)
    t0 = time.perf_counter()
    info = simulation.start(p, simulation.METHOD_MC, n_iterations=sweeps)
    dt = time.perf_counter() - t0
    state.delete(p)
    o = OracleSystem(spec)
    s = random_spins(NOS, 5)
    c0 = time.perf_counter()
    o.mc(s, 3, temperature=10.0)
    cpu_s = time.perf_counter() - c0
    return {
        "workload": "Metropolis Monte Carlo, SC 128x128x16 (J=1, D=0.2, K=0.05 meV, B=0.5 T), T=10 K, adaptive cone, "
                    "colour-ordered sweeps, FP32",
        "sweeps": int(info.total_iterations), "wall_s": dt, "value": NOS * int(info.total_iterations) / dt,
        "unit": "spin-updates/s",
        "timing": "wall clock of Simulation_MC_Start (host checks between device chunks included)",
        "cpu_baseline": {"value": NOS * 3 / cpu_s, "unit": "spin-updates/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": "3 sweeps of the same lattice (FP64, OpenMP)"},
    }


def htst_spec(L):
    """Skyrmion-collapse system of the reference's solver test (core/test/input/solvers.cfg
    parameters: SC, J=10, Bloch D=6 meV, B=25 T, periodic in-plane) on an L x L lattice."""
    return dict(bravais="sc", n_cells=[L, L, 1], lattice_constant=1.0, mu_s=[2.0], bc=[1, 1, 0],
                field=(25.0, (0, 0, 1)), anisotropy=(0.0, (0, 0, 1)), jij=[10.0], dij=[6.0], dm_chirality=1,
                llg=dict(dt=1e-3, damping=0.3, temperature=0.0, force_convergence=1e-10),
                gneb=dict(spring_constant=1.0, force_convergence=1e-9))


def run_htst(sizes=(16, 32), cpu_size=16):
    """HTST prefactor of skyrmion collapse: FP64 minimum (LBFGS_OSO to 1e-10) and saddle point
    (GNEB, 9 images, VP_OSO + climbing image to 1e-9) prepared on the device, then HTST_Calculate
    (dense: all eigenpairs of both 2N x 2N geodesic Hessians) timed by wall clock; CPU: the oracle's
    HTST (FP64, serial cyclic Jacobi) on the smallest size."""
    from oracle.oracle import OracleSystem
    from spirit_gb300 import chain, configuration, htst, simulation, state, system, transition
    from spirit_gb300.configs import write_config
    import spirit_gb300.parameters.gneb as gneb

    out = {"workload": "HTST of skyrmion collapse, SC L x L periodic, J=10, Bloch D=6 meV, B=25 T; minimum "
                       "LBFGS_OSO to 1e-10, saddle point GNEB (9 images, VP_OSO + climbing image) to 1e-9 meV, "
                       "FP64; dense HTST_Calculate (all eigenpairs of both 2N x 2N geodesic Hessians)",
           "timing": "wall clock of HTST_Calculate (gradients, Hessian assembly, two eigen-decompositions, "
                     "velocities)", "sizes": []}
    for L in sizes:
        spec = htst_spec(L)
        p = state.setup(write_config(spec, os.path.join(tempfile.mkdtemp(), "htst.cfg")), True)
        simulation.set_precision(p, 64)
        configuration.plus_z(p)
        configuration.skyrmion(p, 5, phase=-90)
        simulation.start(p, simulation.METHOD_LLG, simulation.SOLVER_LBFGS_OSO, 200000)
        noi = 9
        chain.image_to_clipboard(p)
        for _ in range(1, noi):
            chain.insert_image_after(p)
        configuration.plus_z(p, idx_image=noi - 1)
        transition.homogeneous(p, 0, noi - 1)
        simulation.start(p, simulation.METHOD_GNEB, simulation.SOLVER_VP_OSO, 5000)
        gneb.set_image_type_automatically(p)
        simulation.start(p, simulation.METHOD_GNEB, simulation.SOLVER_VP_OSO, 400000)
        E = [system.get_energy_fp64(p, i) for i in range(noi)]
        sp = int(np.argmax(E[1:-1])) + 1
        smin = np.array(system.get_spin_directions(p, 0))
        ssp = np.array(system.get_spin_directions(p, sp))
        htst.calculate(p, 0, sp, 0, False)  # warm-up (module load, allocations)
        t0 = time.perf_counter()
        pf = htst.calculate(p, 0, sp, 0, False)
        dt = time.perf_counter() - t0
        r = htst.get_result_fp64(p)
        entry = {"L": L, "n_spins": L * L, "matrix_order": 2 * L * L, "status": r["status"], "wall_s": dt,
                 "prefactor": r["prefactor"], "Omega_0": r["Omega_0"], "s": r["s"],
                 "barrier_meV": E[sp] - E[0], "max_torque_gneb": simulation.get_max_torque_norm(p)}
        state.delete(p)
        if L == cpu_size:
            o = OracleSystem(spec)
            c0 = time.perf_counter()
            ro = o.htst(smin, ssp, n_keep=0)
            cdt = time.perf_counter() - c0
            entry["cpu_baseline"] = {"value": cdt, "unit": "s", "cores": 1, "kind": "port",
                                     "sample": "the oracle's dense HTST of the same pair (serial Jacobi)",
                                     "prefactor": ro["prefactor"], "status": ro["status"]}
        out["sizes"].append(entry)
    return out


def run_gb300(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from spirit_gb300 import build as _b

    if not os.path.exists(os.path.join(ROOT, "spirit_gb300", "libspirit_gb300.so")):
        _b.build()
    from oracle.oracle import random_spins
    from spirit_gb300 import simulation, state, system
    from spirit_gb300.configs import write_config
    from spirit_gb300.spiritlib import fn

    profile = fn("Simulation_Profile_Steps", [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong,
                                              ctypes.c_void_p, ctypes.c_longlong, ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int])
    launch = fn("Simulation_Launch_Steps", [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int])
    kps = fn("Simulation_Get_Kernels_Per_Step", [ctypes.c_void_p, ctypes.c_int, ctypes.c_int], ctypes.c_int)
    cfg = write_config(SPEC, os.path.join(tempfile.mkdtemp(), "bench.cfg"))
    p = state.setup(cfg, True)
    system.get_spin_directions(p)[:] = random_spins(NOS, 1 + rank)
    simulation.set_precision(p, 32)
    stream = torch.cuda.Stream()
    simulation.set_stream(p, stream.cuda_stream)
    flush = torch.empty(512 * 2**20, dtype=torch.uint8, device="cuda")
    clean = torch.ones(128 * 2**20, dtype=torch.float32, device="cuda")

    def flush_l2(k):
        flush.fill_(k & 0xFF)
        return clean.sum()
    # --- device-timed steps (inputs resident in HBM)
    simulation.start(p, simulation.METHOD_LLG, simulation.SOLVER_HEUN, 10**9, -1, True)
    launch(p, args.warmup, -1, -1)
    stream.synchronize()
    e0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    e1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush_l2(k)
                e0[k].record(stream)
            launch(p, 1, -1, -1)
            e1[k].record(stream)
        stream.synchronize()
    torch.cuda.synchronize()
    ms = reduce_max(sum(a.elapsed_time(b) for a, b in zip(e0, e1)), world)
    n_kernels = kps(p, -1, -1)
    tun = (ctypes.c_int * 16)()
    ntun = fn("Simulation_Get_Tuning", [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int], ctypes.c_int)(p, tun, 16, -1, -1)
    tuned = dict(zip(["stage_spins_per_thread", "fft_a_lines", "fft_a_threads", "fft_b_lines", "fft_b_threads",
                      "fft_c_columns", "fft_c_threads", "fused_bc", "bc_cluster", "bc_threads", "ddi",
                      "row_fused_stages", "tma_stage", "compensated_state"],
                     [int(tun[k]) for k in range(ntun)]))
    rows = bool(tuned.get("row_fused_stages", 0))
    value = NOS * args.steps * world / (ms / 1000.0)
    if args.profile_step:
        # one more step inside a profiler range: `ncu --profile-from-start off` captures exactly
        # the kernels of one Heun step with the tuned shapes
        stream.synchronize()
        torch.cuda.profiler.start()
        launch(p, 1, -1, -1)
        stream.synchronize()
        torch.cuda.profiler.stop()
    # --- per-kernel durations (CUDA events between launches, L2 flushed before every step)
    kms = (ctypes.c_double * 16)()
    kcount = (ctypes.c_int * 16)()
    profile(p, args.steps, ctypes.c_void_p(flush.data_ptr()), flush.numel(), ctypes.c_void_p(clean.data_ptr()),
            clean.numel() * 4, kms, kcount, -1, -1)
    stream.synchronize()
    per = {KERNELS[i]: (kms[i], kcount[i]) for i in range(len(KERNELS)) if kcount[i] > 0 and KERNELS[i]}
    total = sum(v[0] for v in per.values())
    dom = max(per, key=lambda k: per[k][0])
    avg_ms = per[dom][0] / per[dom][1]
    if dom == "stage":
        # both Heun stages share the kernel name; average their algorithmic bytes
        alg = 0.5 * (algorithmic_bytes("stage", 1, rows) + algorithmic_bytes("stage", 2, rows))
    else:
        alg = algorithmic_bytes(dom, 1)
    peak, peak_kind = measured_peaks()
    achieved = alg / (avg_ms * 1e-3) / 1e9
    # --- end to end through the public API: every step uploads the host spin buffer (H2D),
    # runs one Heun step and brings the spins back (D2H) -- Simulation_SingleShot semantics
    simulation.stop(p)
    simulation.set_stream(p, None)
    simulation.start(p, simulation.METHOD_LLG, simulation.SOLVER_HEUN, 10**9, -1, True)
    for _ in range(args.warmup):
        simulation.single_shot(p)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        simulation.single_shot(p)
    e2e_s = time.perf_counter() - t0
    simulation.stop(p)
    state.delete(p)
    ddi_ms = None
    if all(k in per for k in ("fft_pass_a", "fft_pass_a_inv_c2r")) and per["fft_pass_a"][1] > 0:
        ddi_ms = sum(per[k][0] for k in ("fft_pass_a", "fft_pass_b", "fft_pass_c_tensor", "fft_pass_b_inv",
                                          "fft_pass_a_inv_c2r", "fft_pass_bc_tensor") if k in per) / per["fft_pass_a"][1]
    cufft = cufft_comparison(ddi_ms) if rank == 0 and args.cufft else None
    accuracy = c2_accuracy() if rank == 0 and args.accuracy else None
    batched = run_batched_vs_plain(max(20, args.steps), max(3, args.warmup)) if args.batched else None
    batched_ddi = (run_batched_vs_plain(max(20, args.steps), max(3, args.warmup), ddi=True)
                   if args.batched and args.batched_ddi else None)
    gneb_line = run_gneb() if args.gneb and rank == 0 else None
    adj_line = run_adjoint() if args.adjoint and rank == 0 else None
    mc_line = run_mc() if args.mc and rank == 0 else None
    htst_line = run_htst() if args.htst and rank == 0 else None
    if rank != 0:
        return
    cpu = cpu_baseline() if world == 1 else None
    line = {
        "metric": METRIC, "value": value, "unit": "spin-updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded random spins)", "config": CONFIG,
        "e2e": {"value": NOS * args.steps / e2e_s, "unit": "spin-updates/s",
                "h2d_bytes_per_step": NOS * 3 * 8, "d2h_bytes_per_step": NOS * 3 * 8},
        "gpu_launches": n_kernels * args.steps,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": profiled_traffic(dom) if not rows else None,
                     "algorithmic_bytes_per_launch": alg, "avg_launch_ms": avg_ms},
        "kernel_share": {k: round(v[0] / total, 4) for k, v in per.items()},
        "autotuned": tuned,
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }
    if cufft is not None:
        line["cufft_comparison"] = cufft
    # verbose sub-measurements first, the metric's own numbers (accuracy, batched vs plain) last
    if batched is not None or batched_ddi is not None:
        line["batched_workloads"] = {k: v["workload"] + "; plain: " + v["plain"]
                                     for k, v in (("batched", batched), ("batched_ddi", batched_ddi)) if v}
    if gneb_line is not None:
        line["gneb"] = gneb_line
    if adj_line is not None:
        line["adjoint"] = adj_line
    if mc_line is not None:
        line["mc"] = mc_line
    if htst_line is not None:
        line["htst"] = htst_line
    if accuracy is not None:
        line["accuracy"] = accuracy
    for key, v in (("batched", batched), ("batched_ddi", batched_ddi)):
        if v is not None:
            line[key] = compact_batched(v)
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-batched", dest="batched", action="store_false",
                    help="skip the 256-system batched-vs-plain measurement")
    ap.add_argument("--no-gneb", dest="gneb", action="store_false",
                    help="skip the 32-image GNEB measurement")
    ap.add_argument("--only-gneb", action="store_true", help="run and print only the GNEB measurement")
    ap.add_argument("--no-adjoint", dest="adjoint", action="store_false", help="skip the adjoint measurement")
    ap.add_argument("--no-mc", dest="mc", action="store_false", help="skip the Monte Carlo measurement")
    ap.add_argument("--no-htst", dest="htst", action="store_false", help="skip the HTST measurement")
    ap.add_argument("--no-cufft", dest="cufft", action="store_false", help="skip the cuFFT timing comparison")
    ap.add_argument("--no-accuracy", dest="accuracy", action="store_false",
                    help="skip the FP32-vs-oracle accuracy run of the headline workload")
    ap.add_argument("--profile-step", action="store_true",
                    help="run one extra step inside a CUDA profiler range (for ncu --profile-from-start off)")
    ap.add_argument("--no-batched-ddi", dest="batched_ddi", action="store_false",
                    help="skip the dipolar variant of the 256-system batched measurement")
    ap.add_argument("--only-batched-ddi", action="store_true",
                    help="run and print only the dipolar batched-vs-plain measurement")
    ap.add_argument("--only-htst", action="store_true", help="run and print only the HTST measurement")
    ap.add_argument("--only-adjoint", action="store_true", help="run and print only the adjoint measurement")
    ap.add_argument("--systems", type=int, default=256,
                    help="--only-batched / --only-batched-ddi: the first N systems of the ensemble (profiling)")
    ap.add_argument("--only-batched", action="store_true",
                    help="run and print only the 256-system batched-vs-plain measurement (profiling)")
    args = ap.parse_args()
    if args.only_adjoint:
        import torch

        torch.cuda.set_device(0)
        print(json.dumps(run_adjoint()))
        return
    if args.only_batched_ddi:
        import torch

        torch.cuda.set_device(0)
        prof = args.profile_step  # profiling: the batched path alone
        print(json.dumps(run_batched_vs_plain(max(20, args.steps), max(3, args.warmup), plain=not prof,
                                              check=not prof, ddi=True, profile_step=prof, n_systems=args.systems)))
        return
    if args.only_htst:
        import torch

        torch.cuda.set_device(0)
        print(json.dumps(run_htst()))
        return
    if args.only_gneb:
        import torch

        torch.cuda.set_device(0)
        print(json.dumps(run_gneb()))
        return
    if args.only_batched:
        import torch

        torch.cuda.set_device(0)
        print(json.dumps(run_batched_vs_plain(args.steps, args.warmup, plain=False, check=False,
                                              profile_step=args.profile_step, n_systems=args.systems)))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
