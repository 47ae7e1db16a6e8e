"""Thread sweep of the CPU baselines on the dipolar bench system (SC 128x128x16, stochastic Heun at
T = 10 K, DDI FFT zero-padded along c): the reference itself (oracle/_ref/golden_harness, Spirit's
own OpenMP FP64 path with kissFFT, compiled from its sources by oracle/ref/Makefile) against the
oracle port (oracle/, FP64, OpenMP), each at OMP_NUM_THREADS = 1, 2, 4, ... up to the host's cores.
Times Simulation_LLG_Start alone (reference) and the oracle's LLG call alone (port); set-up and
the dipole-tensor precompute are excluded from both.  Prints one JSON line per run.

    python oracle/ref/sweep_c2.py [--steps N] [--threads 1,2,4,8]

Needs the reference build (present only where the reference sources are).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

PORT = r"""
import sys, time, json
sys.path.insert(0, %r)
import bench
from oracle.oracle import OracleSystem, random_spins
o = OracleSystem(bench.SPEC)
s = random_spins(bench.NOS, 1)
t0 = time.perf_counter()
o.llg(s, "Heun", %d, dt=5e-4, damping=0.1, temperature=10.0, seed=2)
print(json.dumps({"seconds": time.perf_counter() - t0}))
"""


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--threads", default=None)
    args = ap.parse_args()
    import bench
    from oracle.oracle import random_spins
    from spirit_gb300.configs import write_config

    tmp = tempfile.mkdtemp()
    cfg = write_config(bench.SPEC, os.path.join(tmp, "c2.cfg"))
    sp = os.path.join(tmp, "spins.bin")
    random_spins(bench.NOS, 1).tofile(sp)
    harness = os.path.join(ROOT, "oracle", "_ref", "golden_harness")
    ncpu = os.cpu_count()
    threads = [int(t) for t in args.threads.split(",")] if args.threads else \
        [t for t in (1, 2, 4, 8, 16, 32, 64) if t <= ncpu]
    for t in threads:
        env = dict(os.environ, OMP_NUM_THREADS=str(t))
        r = subprocess.run([harness, "llgtime", cfg, sp, "3", str(args.steps)], cwd=tmp, env=env,
                           capture_output=True, text=True, check=True)
        sec = float(r.stdout.split("seconds")[1])
        print(json.dumps({"impl": "reference", "threads": t, "steps": args.steps, "seconds": sec,
                          "spin_updates_per_s": bench.NOS * args.steps / sec}), flush=True)
        r = subprocess.run([sys.executable, "-c", PORT % (ROOT, args.steps)], env=env, capture_output=True, text=True,
                           check=True)
        sec = json.loads(r.stdout.strip().splitlines()[-1])["seconds"]
        print(json.dumps({"impl": "port", "threads": t, "steps": args.steps, "seconds": sec,
                          "spin_updates_per_s": bench.NOS * args.steps / sec}), flush=True)


if __name__ == "__main__":
    main()
